// Internal types of libstokes_gb300: the slot layout of one multigrid level, device
// vector types and error plumbing.
//
// Slot layout. A level with n cells per axis stores every unknown of cell (i,j,k) and of
// its three "left" faces in one slot: slot (i,j,k) holds p(i,j,k), u = x-face (i,j,k),
// v = y-face (i,j,k), w = z-face (i,j,k). Logical indices run over [0, n] per axis (the
// extra plane holds the far boundary faces); a one-slot halo surrounds the box, so every
// 13-point stencil access of a slot in [0,n]^3 stays inside the allocation without
// bounds checks. Padded dims: sx = sy = n + 3, sz = n + 4 (even, so FP64 rows start on
// 32-byte boundaries). Unknowns that do not exist (p at i == n, u at j == n, the halo)
// hold 0 and are marked fixed in the mask, which is how the reference's padded faces
// behave (stoke/StokeFlowDescriptor3D.cu:37-50).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/stokes_gb300.h"

namespace stg {

// Mask bits per slot: set = fixed (Dirichlet identity row), or not present.
enum : uint8_t { MP = 1, MU = 2, MV = 4, MW = 8, MALL = 15 };

struct alignas(32) d4 {
    double p, u, v, w;
};

struct Geom {
    int n = 0;
    int sx = 0, sy = 0, sz = 0;
    long long nslot = 0;
    // division by m = n + 1 as a multiply-high and shift: with s = ceil(log2 m) and
    // dmul = ceil(2^(31+s) / m) (below 2^32), floor(u dmul / 2^(31+s)) = floor(u / m) for
    // every u < 2^31 (Granlund and Montgomery, "Division by invariant integers using
    // multiplication", 1994, thm. 4.2: dmul m - 2^(31+s) < m <= 2^s). Box indices stay below
    // 1025^3 < 2^31. dmul = 0 (a Geom not built by make) falls back to division.
    unsigned dmul = 0;
    int dsh = 0;  // s - 1
    __host__ __device__ int di() const { return sy * sz; }
    __host__ __device__ int dj() const { return sz; }
    __host__ __device__ int slot(int i, int j, int k) const { return ((i + 1) * sy + (j + 1)) * sz + (k + 1); }
    // slots of the logical box [0,n]^3 enumerated by a flat index t
    __host__ __device__ long long box() const { return (long long)(n + 1) * (n + 1) * (n + 1); }
    __host__ __device__ unsigned div_m(unsigned u) const {
#ifdef __CUDA_ARCH__
        return __umulhi(u, dmul) >> dsh;
#else
        return (unsigned)(((unsigned long long)u * dmul) >> 32) >> dsh;
#endif
    }
    __host__ __device__ void box_ijk(long long t, int& i, int& j, int& k) const {
        const int m = n + 1;
        if (dmul) {
            const unsigned u = (unsigned)t, r = div_m(u), q = div_m(r);
            k = (int)(u - r * (unsigned)m);
            j = (int)(r - q * (unsigned)m);
            i = (int)q;
            return;
        }
        k = (int)(t % m);
        long long r = t / m;
        j = (int)(r % m);
        i = (int)(r / m);
    }
    static Geom make(int n) {
        Geom g;
        g.n = n;
        g.sx = n + 3;
        g.sy = n + 3;
        g.sz = n + 4;
        g.nslot = (long long)g.sx * g.sy * g.sz;
        const unsigned long long m = (unsigned long long)n + 1;
        if (n >= 1 && g.box() < (1ll << 31)) {
            int s = 0;
            while ((1ull << s) < m) s++;
            g.dmul = (unsigned)(((1ull << (31 + s)) + m - 1) / m);
            g.dsh = s - 1;
        }
        return g;
    }
};

// Existence of each unknown kind at logical slot (i,j,k) in [0,n]^3.
__host__ __device__ inline bool cell_ok(int n, int i, int j, int k) { return i < n && j < n && k < n; }
__host__ __device__ inline bool face_ok(int n, int d, int i, int j, int k) {
    return (d == 0 ? i <= n : i < n) && (d == 1 ? j <= n : j < n) && (d == 2 ? k <= n : k < n);
}
__host__ __device__ inline uint8_t invalid_bits(int n, int i, int j, int k) {
    uint8_t b = 0;
    if (!cell_ok(n, i, j, k)) b |= MP;
    if (!face_ok(n, 0, i, j, k)) b |= MU;
    if (!face_ok(n, 1, i, j, k)) b |= MV;
    if (!face_ok(n, 2, i, j, k)) b |= MW;
    return b;
}

// Reference blocked layout index math (common_cpx/grid3D.cu:24-105), used by the
// LinearMapping adapters to translate between the reference vectors and the slots.
struct Blocked {
    int n;
    __host__ __device__ long long cell_size() const { return (long long)n * n * n; }
    __host__ __device__ long long face_size() const { return (long long)(n + 4) * n * n; }
    __host__ __device__ long long size() const { return cell_size() + 3 * face_size(); }
    __host__ __device__ void ind_cell(long long idx, int& x, int& y, int& z) const {
        int nb = n >> 2;
        int ix = (int)(idx & 3), iy = (int)((idx >> 2) & 3), iz = (int)((idx >> 4) & 3);
        long long b = idx >> 6;
        x = (int)((b % nb) << 2) + ix;
        y = (int)(((b / nb) % nb) << 2) + iy;
        z = (int)((b / nb / nb) << 2) + iz;
    }
    __host__ __device__ void ind_face(long long idx, int d, int& x, int& y, int& z) const {
        int nbx = (n >> 2) + (d == 0), nby = (n >> 2) + (d == 1);
        int a = (int)(idx & 3), b4 = (int)((idx >> 2) & 3), c = (int)((idx >> 4) & 3);
        long long b = idx >> 6;
        int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / nbx / nby);
        x = (bx << 2) + (d == 0 ? c : a);
        y = (by << 2) + (d == 0 ? a : d == 1 ? c : b4);
        z = (bz << 2) + (d == 2 ? c : b4);
    }
};

// ---------------------------------------------------------------- errors
void set_error(const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define STG_CK(call)                                                          \
    do {                                                                      \
        cudaError_t e_ = (call);                                              \
        if (e_ != cudaSuccess) return ::stg::cuda_fail(e_, #call, __FILE__, __LINE__); \
    } while (0)
#define STG_TRY(expr)            \
    do {                         \
        int s_ = (expr);         \
        if (s_ != STG_OK) return s_; \
    } while (0)
// every kernel launch site checks the launch and counts it
void count_launch();
void add_launches(long long k);
#define STG_LAUNCH_CK()            \
    do {                           \
        ::stg::count_launch();     \
        STG_CK(cudaGetLastError()); \
    } while (0)

// One-time per-device state (kernel attributes, device flags) is kept per device ordinal:
// these are properties of a device, and a process may drive several.
constexpr int MAX_DEVICES = 64;
inline int device_slot() {
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= MAX_DEVICES) {
        cudaGetLastError();
        return -1;
    }
    return d;
}

inline unsigned grid_for(long long work, int block) {
    long long g = (work + block - 1) / block;
    return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace stg
