// Coarsest-level direct solve (DirectSolve3D, stoke/StokeLike.cu:374-648) on the GPU.
//
// The dense matrix is read off the same nine probes as the reference: two cell probes
// coloured by (x+y+z+flag) mod 2 and seven face probes coloured by
// (x + 2y + 3z + magic[d] + flag) mod 7, magic = {2,4,5}; each probe image entry is
// stored at the column the colouring rule assigns to its row (:431-603). Cell-cell
// entries are never recorded (as in the reference); with `closed` the pressure block
// gets +1 everywhere (:605-608). Unknowns that exist only as padding in the reference
// layout are identity rows decoupled from the rest, so the dense system here keeps the
// unknowns that exist. It is inverted once per set-up by Gauss-Jordan elimination with
// partial pivoting on [A | I] (double-buffered in L2; all pivot steps in one cooperative
// launch with a grid-wide barrier between them), and the inverse is applied as a GEMV
// inside each V-cycle.
#include <cooperative_groups.h>

#include <vector>

#include "kernels.h"
#include "stencil.cuh"

namespace stg {

namespace {

constexpr int TPB = 256;

__global__ void k_probe(Geom g, int kind, int flag, d4* __restrict__ probe) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= g.box()) return;
    int i, j, k;
    g.box_ijk(t, i, j, k);
    const int n = g.n;
    const int magic[3] = {2, 4, 5};
    double v[4] = {0, 0, 0, 0};
    if (kind == 0) {
        if (cell_ok(n, i, j, k)) v[0] = ((i + j + k + flag) % 2 == 0) ? 1.0 : 0.0;
    } else {
        for (int d = 0; d < 3; d++)
            if (face_ok(n, d, i, j, k)) v[d + 1] = ((i + 2 * j + 3 * k + magic[d] + flag) % 7 == 0) ? 1.0 : 0.0;
    }
    store4(probe, g.slot(i, j, k), v[0], v[1], v[2], v[3]);
}

// Scatter one probe image into the dense matrix (column-major, nd x nd).
__global__ void k_scatter(Geom g, int kind, int flag, int nd, const int* __restrict__ slot_of, const int* __restrict__ comp_of,
                          const int* __restrict__ dense_of, const d4* __restrict__ image, double* __restrict__ A) {
    int row = blockIdx.x * TPB + threadIdx.x;
    if (row >= nd) return;
    const int n = g.n;
    int s = slot_of[row], c = comp_of[row];
    // logical coordinates of the slot
    int k = s % g.sz - 1, r = s / g.sz;
    int j = r % g.sy - 1, i = r / g.sy - 1;
    double val = reinterpret_cast<const double*>(image)[4ll * s + c];
    int ci = -1, cj = 0, ck = 0, cc = 0;
    if (kind == 0) {
        if (c == 0) return;  // cell rows are not read from the cell probes
        int d = c - 1;
        ci = i;
        cj = j;
        ck = k;
        if ((i + j + k + flag) % 2 == 1) {
            if (d == 0) ci--;
            if (d == 1) cj--;
            if (d == 2) ck--;
        }
        if (!(ci >= 0 && cj >= 0 && ck >= 0 && cell_ok(n, ci, cj, ck))) return;
        cc = 0;
    } else {
        const int magic[3] = {2, 4, 5};
        ci = i;
        cj = j;
        ck = k;
        if (c == 0) {
            switch ((i + 2 * j + 3 * k + flag) % 7) {
                case 1: cc = 2; cj++; break;
                case 2: cc = 3; break;
                case 3: cc = 2; break;
                case 4: cc = 1; ci++; break;
                case 5: cc = 1; break;
                case 6: cc = 3; ck++; break;
                default: return;
            }
        } else {
            int d = c - 1;
            cc = c;
            switch ((i + 2 * j + 3 * k + magic[d] + flag) % 7) {
                case 1: ci--; break;
                case 2: cj--; break;
                case 3: ck--; break;
                case 4: ck++; break;
                case 5: cj++; break;
                case 6: ci++; break;
                default: break;
            }
        }
        // a column outside the existing unknowns is a padding column of the reference layout
        if (ci < 0 || cj < 0 || ck < 0 || !face_ok(n, cc - 1, ci, cj, ck)) return;
    }
    int col = dense_of[4 * g.slot(ci, cj, ck) + cc];
    if (col < 0) return;
    A[(long long)row * 2 * nd + col] = val;
}

__global__ void k_closed(int nd, const int* __restrict__ comp_of, double* __restrict__ A) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= (long long)nd * nd) return;
    int row = (int)(t / nd), col = (int)(t % nd);
    if (comp_of[row] == 0 && comp_of[col] == 0) A[(long long)row * 2 * nd + col] += 1.0;
}

// [A | I]: zero the left half (filled by the probes), identity on the right half
__global__ void k_aug_init(int nd, double* __restrict__ A) {
    long long t = (long long)blockIdx.x * TPB + threadIdx.x;
    if (t >= 2ll * nd * nd) return;
    int row = (int)(t / (2 * nd)), col = (int)(t % (2 * nd));
    A[t] = (col >= nd && col - nd == row) ? 1.0 : 0.0;
}

// Pivot of column k among rows k..nd-1 of the row-major nd x 2nd matrix (largest |a|, the
// first on ties, as LAPACK), found by every block; loads through L2 (the cooperative
// kernel rewrites the buffers during its launch).
__device__ __forceinline__ int gj_pivot(int nd, int k, const double* in) {
    __shared__ double sv[TPB / 32];
    __shared__ int si[TPB / 32];
    __shared__ int sp;
    const int W = 2 * nd;
    double best = -1.0;
    int bi = nd;
    for (int r = k + threadIdx.x; r < nd; r += TPB) {
        const double a = fabs(__ldcg(in + (long long)r * W + k));
        if (a > best || (a == best && r < bi)) {
            best = a;
            bi = r;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
        }
    }
    if ((threadIdx.x & 31) == 0) {
        sv[threadIdx.x >> 5] = best;
        si[threadIdx.x >> 5] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = -1.0;
        int ii = nd;
        for (int w = 0; w < TPB / 32; w++)
            if (sv[w] > b || (sv[w] == b && si[w] < ii)) {
                b = sv[w];
                ii = si[w];
            }
        sp = ii;
    }
    __syncthreads();
    return sp;
}

// One Gauss-Jordan pivot step, rows row0, row0 + rstep, ... of the output: row k <- row
// p / a_pk, row p <- row k - a_kk row k', other rows i <- row i - a_ik row k'. The
// reciprocal of the pivot is formed once per block (an FP64 division per thread costs
// more than the row on GB300's FP64 pipe).
__device__ __forceinline__ void gj_rows(int nd, int k, int p, const double* in, double* out, int* info, int row0, int rstep) {
    __shared__ double s_inv;
    const int W = 2 * nd;
    const double piv = __ldcg(in + (long long)p * W + k);
    if (threadIdx.x == 0) s_inv = piv != 0.0 ? 1.0 / piv : 0.0;
    __syncthreads();
    const double inv = s_inv;
    for (int row = row0; row < nd; row += rstep) {
        if (piv == 0.0) {
            if (row == 0 && threadIdx.x == 0 && *info == 0) *info = k + 1;
            for (int c = threadIdx.x; c < W; c += TPB) out[(long long)row * W + c] = __ldcg(in + (long long)row * W + c);
            continue;
        }
        const int src = row == k ? p : (row == p ? k : row);
        const double f = row == k ? 0.0 : __ldcg(in + (long long)src * W + k);
        for (int c = threadIdx.x; c < W; c += TPB) {
            const double pr = __ldcg(in + (long long)p * W + c) * inv;
            out[(long long)row * W + c] = row == k ? pr : __ldcg(in + (long long)src * W + c) - f * pr;
        }
    }
    __syncthreads();  // s_inv and the pivot's shared words are rewritten by the next step
}

// One pivot step per launch (block b handles row b); the fallback where a cooperative
// launch is unavailable.
__global__ void __launch_bounds__(TPB) k_gj_step(int nd, int k, const double* in, double* out, int* info) {
    const int p = gj_pivot(nd, k, in);
    gj_rows(nd, k, p, in, out, info, blockIdx.x, nd);
}

// All nd pivot steps in one cooperative launch, a grid-wide barrier between them (the
// launch gaps of nd dependent kernels were most of the set-up time): the operations of
// k_gj_step in the same order, so the same inverse bit for bit. Step k reads buffer k mod
// 2 and writes the other.
__global__ void __launch_bounds__(TPB) k_gj_all(int nd, double* a, double* b, int* info) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    for (int k = 0; k < nd; k++) {
        const double* in = (k & 1) ? b : a;
        double* out = (k & 1) ? a : b;
        const int p = gj_pivot(nd, k, in);
        gj_rows(nd, k, p, in, out, info, blockIdx.x, gridDim.x);
        grid.sync();
    }
}

template <class V>
__device__ __forceinline__ double comp_value(const V* r, int s, int c);
template <>
__device__ __forceinline__ double comp_value<float4>(const float4* r, int s, int c) {
    return (double)reinterpret_cast<const float*>(r)[4ll * s + c];
}
template <>
__device__ __forceinline__ double comp_value<d4>(const d4* r, int s, int c) {
    return reinterpret_cast<const double*>(r)[4ll * s + c];
}

template <class V>
__global__ void k_gather(int nd, const int* __restrict__ slot_of, const int* __restrict__ comp_of, const V* __restrict__ r,
                         double* __restrict__ rd) {
    int q = blockIdx.x * TPB + threadIdx.x;
    if (q < nd) rd[q] = comp_value<V>(r, slot_of[q], comp_of[q]);
}

// one warp per row: x[row] = sum_c Ainv[row, c] rd[c], scattered into the slot vector
template <class T>
__global__ void k_gemv(int nd, const double* __restrict__ Ainv, int ld, const double* __restrict__ rd,
                       const int* __restrict__ slot_of, const int* __restrict__ comp_of, T* __restrict__ x) {
    int row = (blockIdx.x * TPB + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (row >= nd) return;
    double s = 0;
    for (int c = lane; c < nd; c += 32) s += Ainv[(long long)row * ld + c] * rd[c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[4ll * slot_of[row] + comp_of[row]] = (T)s;
}

}  // namespace

int dense_init(DenseCoarse& D, const Geom& g) {
    std::vector<int> slot_of, comp_of, dense_of((size_t)g.nslot * 4, -1);
    const int n = g.n;
    for (int i = 0; i <= n; i++)
        for (int j = 0; j <= n; j++)
            for (int k = 0; k <= n; k++) {
                int s = g.slot(i, j, k);
                for (int c = 0; c < 4; c++) {
                    bool ok = c == 0 ? cell_ok(n, i, j, k) : face_ok(n, c - 1, i, j, k);
                    if (!ok) continue;
                    dense_of[4 * (size_t)s + c] = (int)slot_of.size();
                    slot_of.push_back(s);
                    comp_of.push_back(c);
                }
            }
    D.nd = (int)slot_of.size();
    size_t nd = D.nd;
    STG_CK(cudaMalloc(&D.slot_of, sizeof(int) * nd));
    STG_CK(cudaMalloc(&D.comp_of, sizeof(int) * nd));
    STG_CK(cudaMalloc(&D.dense_of, sizeof(int) * dense_of.size()));
    STG_CK(cudaMalloc(&D.A, sizeof(double) * 2 * nd * nd));
    STG_CK(cudaMalloc(&D.Ainv, sizeof(double) * 2 * nd * nd));
    STG_CK(cudaMalloc(&D.piv, sizeof(int) * nd));
    STG_CK(cudaMalloc(&D.info, sizeof(int)));
    STG_CK(cudaMalloc(&D.probe, sizeof(d4) * g.nslot));
    STG_CK(cudaMalloc(&D.image, sizeof(d4) * g.nslot));
    STG_CK(cudaMalloc(&D.rd, sizeof(double) * nd));
    STG_CK(cudaMemcpy(D.slot_of, slot_of.data(), sizeof(int) * nd, cudaMemcpyHostToDevice));
    STG_CK(cudaMemcpy(D.comp_of, comp_of.data(), sizeof(int) * nd, cudaMemcpyHostToDevice));
    STG_CK(cudaMemcpy(D.dense_of, dense_of.data(), sizeof(int) * dense_of.size(), cudaMemcpyHostToDevice));
    STG_CK(cudaMemset(D.probe, 0, sizeof(d4) * g.nslot));
    STG_CK(cudaMemset(D.image, 0, sizeof(d4) * g.nslot));
    return STG_OK;
}

void dense_free(DenseCoarse& D) {
    cudaFree(D.slot_of);
    cudaFree(D.comp_of);
    cudaFree(D.dense_of);
    cudaFree(D.A);
    cudaFree(D.Ainv);
    cudaFree(D.piv);
    cudaFree(D.info);
    cudaFree(D.probe);
    cudaFree(D.image);
    cudaFree(D.rd);
    D = DenseCoarse();
}

int op64v(cudaStream_t st, const Geom& g, const d4* x, const uint8_t* m, const d4* P, const d4* V, const d4* b, d4* out,
          int mode, double* part, int* nb_out);

int dense_setup_v(cudaStream_t st, DenseCoarse& D, const Geom& g, const d4* V, const uint8_t* m, const d4* P64, int closed,
                  const std::function<int(double*, int)>& extra) {
    const int nd = D.nd;
    k_aug_init<<<grid_for(2ll * nd * nd, TPB), TPB, 0, st>>>(nd, D.A);
    STG_LAUNCH_CK();
    for (int kind = 0; kind < 2; kind++) {
        int nflags = kind == 0 ? 2 : 7;
        for (int f = 0; f < nflags; f++) {
            k_probe<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, kind, f, D.probe);
            STG_LAUNCH_CK();
            STG_TRY(op64v(st, g, D.probe, m, P64, V, nullptr, D.image, 0, nullptr, nullptr));
            k_scatter<<<grid_for(nd, TPB), TPB, 0, st>>>(g, kind, f, nd, D.slot_of, D.comp_of, D.dense_of, D.image, D.A);
            STG_LAUNCH_CK();
        }
    }
    if (closed) {
        k_closed<<<grid_for((long long)nd * nd, TPB), TPB, 0, st>>>(nd, D.comp_of, D.A);
        STG_LAUNCH_CK();
    }
    if (extra) STG_TRY(extra(D.A, nd));
    return gj_invert(st, nd, D.A, D.Ainv, D.info, &D.inv, true);
}

int dense_setup(cudaStream_t st, DenseCoarse& D, const Geom& g, double vol, const uint8_t* m, const d4* P64, int closed,
                bool invert) {
    const int nd = D.nd;
    k_aug_init<<<grid_for(2ll * nd * nd, TPB), TPB, 0, st>>>(nd, D.A);
    STG_LAUNCH_CK();
    for (int kind = 0; kind < 2; kind++) {
        int nflags = kind == 0 ? 2 : 7;
        for (int f = 0; f < nflags; f++) {
            k_probe<<<grid_for(g.box(), TPB), TPB, 0, st>>>(g, kind, f, D.probe);
            STG_LAUNCH_CK();
            STG_TRY(op64(st, g, vol, D.probe, m, P64, nullptr, D.image, 0, nullptr, nullptr));
            k_scatter<<<grid_for(nd, TPB), TPB, 0, st>>>(g, kind, f, nd, D.slot_of, D.comp_of, D.dense_of, D.image, D.A);
            STG_LAUNCH_CK();
        }
    }
    if (closed) {
        k_closed<<<grid_for((long long)nd * nd, TPB), TPB, 0, st>>>(nd, D.comp_of, D.A);
        STG_LAUNCH_CK();
    }
    return invert ? gj_invert(st, nd, D.A, D.Ainv, D.info, &D.inv) : STG_OK;
}

int gj_invert(cudaStream_t st, int nd, double* a, double* b, int* info, const double** inv, bool coop) {
    STG_CK(cudaMemsetAsync(info, 0, sizeof(int), st));
    if (coop) {
        // one block per SM at most (fewer blocks, a cheaper grid barrier), within what can
        // be co-resident
        int dev = 0, sms = 0, per_sm = 0;
        STG_CK(cudaGetDevice(&dev));
        STG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        STG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gj_all, TPB, 0));
        if (per_sm >= 1 && sms >= 1) {
            const int g = nd < sms ? nd : sms;
            void* args[] = {&nd, &a, &b, &info};
            STG_CK(cudaLaunchCooperativeKernel((const void*)k_gj_all, dim3((unsigned)g), dim3(TPB), args, 0, st));
            add_launches(1);
            *inv = (nd & 1) ? b + nd : a + nd;  // step nd-1 wrote buffer nd mod 2
            return STG_OK;
        }
    }
    for (int k = 0; k < nd; k++) {
        k_gj_step<<<nd, TPB, 0, st>>>(nd, k, a, b, info);
        STG_LAUNCH_CK();
        double* t = a;
        a = b;
        b = t;
    }
    *inv = a + nd;  // right half of the final buffer, row stride 2 nd
    return STG_OK;
}

int dense_apply32(cudaStream_t st, const DenseCoarse& D, const Geom& g, const float4* r, float4* x) {
    double* rd = D.rd;
    k_gather<float4><<<grid_for(D.nd, TPB), TPB, 0, st>>>(D.nd, D.slot_of, D.comp_of, r, rd);
    STG_LAUNCH_CK();
    STG_CK(cudaMemsetAsync(x, 0, sizeof(float4) * g.nslot, st));
    k_gemv<float><<<grid_for(32ll * D.nd, TPB), TPB, 0, st>>>(D.nd, D.inv, 2 * D.nd, rd, D.slot_of, D.comp_of,
                                                              reinterpret_cast<float*>(x));
    STG_LAUNCH_CK();
    return STG_OK;
}

int dense_apply64(cudaStream_t st, const DenseCoarse& D, const Geom& g, const d4* r, d4* x) {
    double* rd = D.rd;
    k_gather<d4><<<grid_for(D.nd, TPB), TPB, 0, st>>>(D.nd, D.slot_of, D.comp_of, r, rd);
    STG_LAUNCH_CK();
    STG_CK(cudaMemsetAsync(x, 0, sizeof(d4) * g.nslot, st));
    k_gemv<double><<<grid_for(32ll * D.nd, TPB), TPB, 0, st>>>(D.nd, D.inv, 2 * D.nd, rd, D.slot_of, D.comp_of,
                                                                reinterpret_cast<double*>(x));
    STG_LAUNCH_CK();
    return STG_OK;
}

}  // namespace stg
