// Allocation-free optimality-criteria update (stg_oc_update_noalloc).
//
// Who needs it: callers that cannot call cudaMalloc - host applications that reserve
// the whole GPU for their own memory pool up front, plugins running under another
// framework's allocator budget, and latency-sensitive design loops that cannot afford
// the device-wide synchronisation that cudaMalloc/cudaFree imply. They pass their own
// device arrays for the design, the sensitivity and the result; the only scratch this
// entry point needs (the per-block partial sums of the volume reduction) lives in the
// fixed array below, which every GPU that loads this library holds until the process
// exits.
//
// The bisection and the volume sums are the ones of stg_oc_update (same kernels'
// arithmetic, same reduction grid and order), with the filter volume weights
// vw_j = sum_i w_ij / W_i formed on the fly instead of being read from a buffer, so both
// entry points return the same design and multiplier.
#include <climits>
#include <cmath>
#include <mutex>

#include "kernels.h"

namespace stg {

namespace {

constexpr int TPB = 256;
constexpr int OC_GRID = 1216;                 // reduction grid (8 x 152 SMs), as stg_oc_update
constexpr int NOALLOC_SCRATCH = 2048;         // doubles: OC_GRID partials + the reduced sum
constexpr long long NOALLOC_MAX_CELLS = 1ll << 30;  // largest design (1024^3 cells)

// Scratch shared by every call on a device. Calls that overlap on the GPU race on it.
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH];

std::mutex g_mu;
double* g_scratch_ptr[256] = {};

// Device address of the scratch on the current device, resolved once per device.
int scratch_on_current_device(double** out) {
    int dev = 0;
    STG_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) {
        set_error("device ordinal %d out of range", dev);
        return STG_E_INVALID;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress", __FILE__, __LINE__);
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[dev];
    return STG_OK;
}

// sum_j w_ij over the cells j of the domain within the hat radius of cell i
__device__ __forceinline__ double hat_wsum(int n, double rmin, int R, int i0, int j0, int k0) {
    double W = 0;
    for (int a = -R; a <= R; a++)
        for (int b = -R; b <= R; b++)
            for (int c = -R; c <= R; c++) {
                int ii = i0 + a, jj = j0 + b, kk = k0 + c;
                if (ii < 0 || jj < 0 || kk < 0 || ii >= n || jj >= n || kk >= n) continue;
                double w = rmin - sqrt((double)(a * a + b * b + c * c));
                if (w > 0) W += w;
            }
    return W;
}

// vw_j = sum_i w_ij / W_i (column sum of the normalised filter)
__device__ __forceinline__ double hat_vw(int n, double rmin, int R, int i, int j, int k) {
    double s = 0;
    for (int a = -R; a <= R; a++)
        for (int b = -R; b <= R; b++)
            for (int c = -R; c <= R; c++) {
                int ii = i + a, jj = j + b, kk = k + c;
                if (ii < 0 || jj < 0 || kk < 0 || ii >= n || jj >= n || kk >= n) continue;
                double w = rmin - sqrt((double)(a * a + b * b + c * c));
                if (w <= 0) continue;
                s += w * 1.0 / hat_wsum(n, rmin, R, ii, jj, kk);
            }
    return s;
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// one bisection probe: x_new(lambda) and per-block partials of sum vw x_new (into scratch)
__global__ void k_oc_noalloc(int n, double rmin, int R, const double* __restrict__ x, const double* __restrict__ dc,
                             double lam, double move, double lo, double hi, double* __restrict__ xnew,
                             double* __restrict__ part) {
    __shared__ double sh[TPB / 32];
    const long long nc = (long long)n * n * n;
    const double inv_n = 1.0 / (double)nc;
    double acc = 0;
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < nc; t += (long long)gridDim.x * TPB) {
        int k = (int)(t % n), j = (int)((t / n) % n), i = (int)(t / ((long long)n * n));
        double vw = hat_vw(n, rmin, R, i, j, k);
        double xi = x[t];
        double dv = vw * inv_n;
        double B = fmax(0.0, -dc[t]) / (dv * lam);
        double xn = xi * sqrt(B);
        xn = fmin(fmin(hi, xi + move), fmax(fmax(lo, xi - move), xn));
        if (xnew) xnew[t] = xn;
        acc += vw * xn;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int w = 0; w < TPB / 32; w++) s += sh[w];
        part[blockIdx.x] = s;
    }
}

}  // namespace

}  // namespace stg

using namespace stg;

extern "C" int stg_oc_update_noalloc(int n, double rmin, const double* d_x, const double* d_dc, double frac, double move,
                                     double lo, double hi, double* d_xnew, double* lambda_out, void* cuda_stream) {
    if (n < 1 || (long long)n * n * n > NOALLOC_MAX_CELLS) {
        set_error("stg_oc_update_noalloc: N = %d outside 1..1024 (design limited to %lld cells)", n, NOALLOC_MAX_CELLS);
        return STG_E_INVALID;
    }
    if (!d_x || !d_dc || !d_xnew || !(rmin > 0)) {
        set_error("stg_oc_update_noalloc: null array or non-positive rmin");
        return STG_E_INVALID;
    }
    double* scratch = nullptr;
    STG_TRY(scratch_on_current_device(&scratch));
    cudaStream_t st = (cudaStream_t)cuda_stream;
    int R = (int)ceil(rmin) - 1;
    if (R < 0) R = 0;
    const long long nc = (long long)n * n * n;
    long long g = (nc + TPB - 1) / TPB;
    if (g > OC_GRID) g = OC_GRID;
    const int grid = (int)g;
    double* part = scratch;                        // OC_GRID partials
    double* sum = scratch + NOALLOC_SCRATCH - 1;   // reduced volume
    double l1 = 0.0, l2 = 1e9, lmid = 0.0, target = frac * (double)nc;
    int steps = 0;
    const double tol = 1e-9;
    auto volume = [&](double lam, double* vol) -> int {
        k_oc_noalloc<<<grid, TPB, 0, st>>>(n, rmin, R, d_x, d_dc, lam, move, lo, hi, nullptr, part);
        STG_LAUNCH_CK();
        STG_TRY(reduce_parts(st, part, grid, sum));
        STG_CK(cudaMemcpyAsync(vol, sum, sizeof(double), cudaMemcpyDeviceToHost, st));
        STG_CK(cudaStreamSynchronize(st));
        return STG_OK;
    };
    // bracket widened by decades while its upper end overshoots the volume (stg_oc_update)
    for (int k = 0; k < 60; k++) {
        double vol = 0;
        STG_TRY(volume(l2, &vol));
        if (vol <= target) break;
        l1 = l2;
        l2 *= 10.0;
    }
    while ((l2 - l1) > tol * (l1 + l2) && steps < 200) {
        lmid = 0.5 * (l1 + l2);
        double vol = 0;
        STG_TRY(volume(lmid, &vol));
        if (vol > target)
            l1 = lmid;
        else
            l2 = lmid;
        steps++;
    }
    lmid = 0.5 * (l1 + l2);
    k_oc_noalloc<<<grid, TPB, 0, st>>>(n, rmin, R, d_x, d_dc, lmid, move, lo, hi, d_xnew, part);
    STG_LAUNCH_CK();
    STG_CK(cudaStreamSynchronize(st));
    if (lambda_out) *lambda_out = lmid;
    return STG_OK;
}
