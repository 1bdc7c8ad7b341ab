// Allocation-free optimality-criteria update (stg_oc_update_noalloc).
//
// Who needs it: callers that cannot call cudaMalloc - host applications that reserve
// the whole GPU for their own memory pool up front, plugins running under another
// framework's allocator budget, and latency-sensitive design loops that cannot afford
// the device-wide synchronisation that cudaMalloc/cudaFree imply. They pass their own
// device arrays for the design, the sensitivity and the result; the only scratch this
// entry point needs (the per-block partial sums of the volume reduction and a small
// table of filter weight sums) lives in the fixed array below, which every GPU that
// loads this library holds until the process exits.
//
// The bisection and the volume sums are the ones of stg_oc_update (same kernels'
// arithmetic, same reduction grid and order), with the filter volume weights
// vw_j = sum_i w_ij / W_i formed on the fly instead of being read from a buffer, so both
// entry points return the same design and multiplier. W_i depends only on how far cell i
// lies from each pair of domain faces (clamped at the filter radius R), so it is read
// from a table of (R+1)^6 classes built once per call, in the summation order of the
// handle's filter; a probe then costs (2R+1)^3 table reads per cell.
#include <climits>
#include <cmath>
#include <mutex>

#include "kernels.h"

namespace stg {

namespace {

constexpr int TPB = 256;
constexpr int OC_GRID = 1216;                 // reduction grid (8 x 152 SMs), as stg_oc_update
constexpr int NOALLOC_MAX_N = 1024;           // largest design: 1024^3 cells
constexpr int NOALLOC_MAX_R = 3;              // largest filter radius index: rmin <= 4
constexpr int NOALLOC_CLASSES = 4096;         // (R+1)^6 weight-sum classes at R = 3
constexpr int NOALLOC_TAB = 343;              // (2R+1)^3 filter weights at R = 3
constexpr int SCR_SUM = OC_GRID;              // reduced volume
constexpr int SCR_WCLASS = 1280;              // start of the class table (256-byte aligned)
constexpr int NOALLOC_SCRATCH = SCR_WCLASS + NOALLOC_CLASSES;  // 5376 doubles = 42 KB

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

// filter weights rmin - |o| for every offset o in [-R, R]^3, formed on the host with
// IEEE sqrt exactly as the handle's filter table
struct WTabNA {
    double w[NOALLOC_TAB];
};

// one axis's class: (how far the cell may reach down, how far up), each clamped at R
__device__ __forceinline__ int axis_class(int i, int n, int R) {
    const int lo = min(i, R), hi = min(n - 1 - i, R);
    return lo * (R + 1) + hi;
}

// W for every class: sum of the positive weights over the offsets the class allows, in
// the loop order of the handle's weight-sum kernel (a, then b, then c), so the sums are
// bit-identical to the ones stg_oc_update reads
__global__ void k_wsum_classes(int R, WTabNA T, double* __restrict__ wc) {
    const int per = (R + 1) * (R + 1);
    const int ncls = per * per * per;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncls) return;
    const int cz = t % per, cy = (t / per) % per, cx = t / (per * per);
    const int xlo = cx / (R + 1), xhi = cx % (R + 1), ylo = cy / (R + 1), yhi = cy % (R + 1), zlo = cz / (R + 1),
              zhi = cz % (R + 1);
    const int D = 2 * R + 1;
    double s = 0;
    for (int a = -R; a <= R; a++)
        for (int b = -R; b <= R; b++)
            for (int c = -R; c <= R; c++) {
                if (a < -xlo || a > xhi || b < -ylo || b > yhi || c < -zlo || c > zhi) continue;
                const double w = T.w[((a + R) * D + (b + R)) * D + (c + R)];
                if (w > 0) s += w;
            }
    wc[t] = s;
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One bisection probe: x_new(lambda) and per-block partials of sum vw x_new (into
// scratch). vw_j = sum_i w_ij / W_i, summed in the handle filter's transpose order. x and
// xnew may be the same array (each element is read before it is written by one thread).
__global__ void k_oc_noalloc(int n, int R, WTabNA T, const double* __restrict__ wclass_g, const double* x,
                             const double* __restrict__ dc, double lam, double move, double lo, double hi, double* xnew,
                             double* __restrict__ part) {
    __shared__ double sh[TPB / 32];
    __shared__ double wcls[NOALLOC_CLASSES];
    const int per = (R + 1) * (R + 1);
    const int ncls = per * per * per;
    for (int c = threadIdx.x; c < ncls; c += TPB) wcls[c] = wclass_g[c];
    __syncthreads();
    const int D = 2 * R + 1;
    const long long nc = (long long)n * n * n;
    const double inv_n = 1.0 / (double)nc;
    double acc = 0;
    for (long long t = (long long)blockIdx.x * TPB + threadIdx.x; t < nc; t += (long long)gridDim.x * TPB) {
        const int k = (int)(t % n), j = (int)((t / n) % n), i = (int)(t / ((long long)n * n));
        double vw = 0;
        for (int a = -R; a <= R; a++) {
            const int ii = i + a;
            if (ii < 0 || ii >= n) continue;
            const int ca = axis_class(ii, n, R) * per * per;
            for (int b = -R; b <= R; b++) {
                const int jj = j + b;
                if (jj < 0 || jj >= n) continue;
                const int cb = ca + axis_class(jj, n, R) * per;
                for (int c = -R; c <= R; c++) {
                    const int kk = k + c;
                    if (kk < 0 || kk >= n) continue;
                    const double w = T.w[((a + R) * D + (b + R)) * D + (c + R)];
                    if (w <= 0) continue;
                    vw += w * 1.0 / wcls[cb + axis_class(kk, n, R)];
                }
            }
        }
        const double xi = x[t];
        const double dv = vw * inv_n;
        const double B = fmax(0.0, -dc[t]) / (dv * lam);
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
    if (n < 1 || n > NOALLOC_MAX_N) {
        set_error("stg_oc_update_noalloc: N = %d outside 1..%d (designs of at most 1024^3 cells)", n, NOALLOC_MAX_N);
        return STG_E_INVALID;
    }
    if (!d_x || !d_dc || !d_xnew) {
        set_error("stg_oc_update_noalloc: null device array");
        return STG_E_INVALID;
    }
    if (!(rmin > 0) || !(rmin <= NOALLOC_MAX_R + 1)) {
        set_error("stg_oc_update_noalloc: filter radius rmin = %g outside (0, %d]", rmin, NOALLOC_MAX_R + 1);
        return STG_E_INVALID;
    }
    double* scratch = nullptr;
    STG_TRY(scratch_on_current_device(&scratch));
    cudaStream_t st = (cudaStream_t)cuda_stream;
    int R = (int)ceil(rmin) - 1;
    if (R < 0) R = 0;
    const int D = 2 * R + 1;
    WTabNA T{};
    for (int a = -R; a <= R; a++)
        for (int b = -R; b <= R; b++)
            for (int c = -R; c <= R; c++) T.w[((a + R) * D + (b + R)) * D + (c + R)] = rmin - sqrt((double)(a * a + b * b + c * c));
    const long long nc = (long long)n * n * n;
    long long g = (nc + TPB - 1) / TPB;
    if (g > OC_GRID) g = OC_GRID;
    const int grid = (int)g;
    double* part = scratch;                 // OC_GRID partials
    double* sum = scratch + SCR_SUM;        // reduced volume
    double* wclass = scratch + SCR_WCLASS;  // W per class
    const int ncls = (R + 1) * (R + 1) * (R + 1) * (R + 1) * (R + 1) * (R + 1);
    k_wsum_classes<<<(ncls + 127) / 128, 128, 0, st>>>(R, T, wclass);
    STG_LAUNCH_CK();
    double l1 = 0.0, l2 = 1e9, lmid = 0.0, target = frac * (double)nc;
    int steps = 0;
    const double tol = 1e-9;
    auto volume = [&](double lam, double* vol) -> int {
        k_oc_noalloc<<<grid, TPB, 0, st>>>(n, R, T, wclass, d_x, d_dc, lam, move, lo, hi, nullptr, part);
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
    k_oc_noalloc<<<grid, TPB, 0, st>>>(n, R, T, wclass, d_x, d_dc, lmid, move, lo, hi, d_xnew, part);
    STG_LAUNCH_CK();
    STG_CK(cudaStreamSynchronize(st));
    if (lambda_out) *lambda_out = lmid;
    return STG_OK;
}
