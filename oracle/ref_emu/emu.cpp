// Host-side stand-in for the CUDA runtime, cuBLAS and cuSOLVER calls the reference's
// solver path makes (see emu.h for the execution model). TEST INFRASTRUCTURE ONLY.
//
// The batched and dense LU factorisations are LAPACK's getrf/getrs semantics (partial
// pivoting by the largest magnitude in the column, row interchanges recorded 1-based,
// unit lower factor), written out from the textbook algorithm.
#include "emu.h"

#include <ucontext.h>

#include <vector>

uint3 threadIdx;
uint3 blockIdx;
dim3 blockDim;
dim3 gridDim;

namespace {

enum class Mode { Fiber, Direct };

struct Fiber {
    ucontext_t ctx;
    std::vector<char> stack;
    uint3 tid;
    bool done = false;
};

constexpr size_t STACK = 256 * 1024;

ucontext_t g_sched;
Fiber* g_cur = nullptr;
const std::function<void()>* g_body = nullptr;
Mode g_mode = Mode::Fiber;
bool g_barrier_seen = false;
std::vector<Fiber> g_pool;

bool env_flag(const char* name) {
    const char* v = getenv(name);
    return v && *v && *v != '0';
}

void fiber_entry() {
    (*g_body)();
    g_cur->done = true;
    swapcontext(&g_cur->ctx, &g_sched);
}

uint3 tid_of(unsigned t, const dim3& b) { return uint3{t % b.x, (t / b.x) % b.y, t / (b.x * b.y)}; }

// runs one block with a fiber per thread; returns whether any thread met a barrier
bool run_block_fibers(unsigned nthr, const dim3& b, bool reverse) {
    if (g_pool.size() < nthr) g_pool.resize(nthr);
    for (unsigned t = 0; t < nthr; t++) {
        Fiber& f = g_pool[t];
        if (f.stack.empty()) f.stack.resize(STACK);
        f.done = false;
        f.tid = tid_of(t, b);
        getcontext(&f.ctx);
        f.ctx.uc_stack.ss_sp = f.stack.data();
        f.ctx.uc_stack.ss_size = f.stack.size();
        f.ctx.uc_link = nullptr;
        makecontext(&f.ctx, fiber_entry, 0);
    }
    g_barrier_seen = false;
    unsigned live = nthr;
    while (live > 0) {
        for (unsigned q = 0; q < nthr; q++) {
            Fiber& f = g_pool[reverse ? nthr - 1 - q : q];
            if (f.done) continue;
            g_cur = &f;
            threadIdx = f.tid;
            swapcontext(&g_sched, &f.ctx);
            if (f.done) live--;
        }
    }
    g_cur = nullptr;
    return g_barrier_seen;
}

}  // namespace

void __syncthreads() {
    if (g_mode == Mode::Direct) {
        fprintf(stderr, "ref_emu: __syncthreads() in a kernel whose first thread met no barrier\n");
        abort();
    }
    g_barrier_seen = true;
    Fiber* f = g_cur;
    swapcontext(&f->ctx, &g_sched);
    threadIdx = f->tid;
}

namespace emu {

void launch(const Cfg& c, const std::function<void()>& body) {
    // EMU_REVERSE=1 runs blocks and the threads of a block in reverse order: a kernel
    // whose result depends on that order relies on scheduling it does not control
    const bool reverse = env_flag("EMU_REVERSE");
    gridDim = c.g;
    blockDim = c.b;
    const unsigned nthr = c.b.x * c.b.y * c.b.z;
    const unsigned nblk = c.g.x * c.g.y * c.g.z;
    if (nthr == 0 || nblk == 0) return;
    g_body = &body;
    bool fibers = true;
    for (unsigned q = 0; q < nblk; q++) {
        const unsigned bi = reverse ? nblk - 1 - q : q;
        blockIdx = uint3{bi % c.g.x, (bi / c.g.x) % c.g.y, bi / (c.g.x * c.g.y)};
        if (fibers) {
            g_mode = Mode::Fiber;
            const bool met = run_block_fibers(nthr, c.b, reverse);
            // a kernel with no barrier in its first block runs the rest as plain calls
            if (!met) fibers = false;
            continue;
        }
        g_mode = Mode::Direct;
        for (unsigned s = 0; s < nthr; s++) {
            threadIdx = tid_of(reverse ? nthr - 1 - s : s, c.b);
            body();
        }
    }
    g_mode = Mode::Fiber;
    g_body = nullptr;
}

}  // namespace emu

// ------------------------------------------------------------------ runtime
cudaError_t cudaMalloc(void** p, size_t bytes) {
    size_t sz = (bytes + 255) / 256 * 256;
    if (sz == 0) sz = 256;
    void* q = aligned_alloc(256, sz);
    if (!q) return cudaErrorMemoryAllocation;
    // device memory starts undefined; EMU_FILL_NAN=1 fills it with NaN so that a read of
    // memory nothing wrote shows up in the results, otherwise it is zeroed
    if (env_flag("EMU_FILL_NAN")) {
        double nan = std::nan("");
        for (size_t i = 0; i + 8 <= sz; i += 8) memcpy(static_cast<char*>(q) + i, &nan, 8);
    } else {
        memset(q, 0, sz);
    }
    *p = q;
    return cudaSuccess;
}
cudaError_t cudaFree(void* p) {
    free(p);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void* dst, const void* src, size_t bytes, cudaMemcpyKind) {
    if (bytes) memmove(dst, src, bytes);
    return cudaSuccess;
}
cudaError_t cudaMemset(void* p, int v, size_t bytes) {
    if (bytes) memset(p, v, bytes);
    return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
cudaError_t cudaGetLastError() { return cudaSuccess; }
cudaError_t cudaPeekAtLastError() { return cudaSuccess; }
cudaError_t cudaDeviceReset() { return cudaSuccess; }
const char* cudaGetErrorName(cudaError_t e) { return e == cudaSuccess ? "cudaSuccess" : "cudaError"; }
const char* cudaGetErrorString(cudaError_t e) { return cudaGetErrorName(e); }

// ------------------------------------------------------------------ dense LU (getrf / getrs)
namespace {

// column-major n x n at a with leading dimension lda; ipiv 1-based; returns info
template <class T>
int getrf(int m, int n, T* a, int lda, int* ipiv) {
    int info = 0;
    const int kmax = std::min(m, n);
    for (int k = 0; k < kmax; k++) {
        int p = k;
        T best = std::fabs(a[k + (size_t)k * lda]);
        for (int i = k + 1; i < m; i++) {
            T v = std::fabs(a[i + (size_t)k * lda]);
            if (v > best) {
                best = v;
                p = i;
            }
        }
        ipiv[k] = p + 1;
        if (a[p + (size_t)k * lda] == T(0)) {
            if (info == 0) info = k + 1;
            continue;
        }
        if (p != k)
            for (int j = 0; j < n; j++) std::swap(a[k + (size_t)j * lda], a[p + (size_t)j * lda]);
        const T inv = T(1) / a[k + (size_t)k * lda];
        for (int i = k + 1; i < m; i++) a[i + (size_t)k * lda] *= inv;
        for (int j = k + 1; j < n; j++) {
            const T akj = a[k + (size_t)j * lda];
            if (akj == T(0)) continue;
            for (int i = k + 1; i < m; i++) a[i + (size_t)j * lda] -= a[i + (size_t)k * lda] * akj;
        }
    }
    return info;
}

template <class T>
void getrs(int n, int nrhs, const T* a, int lda, const int* ipiv, T* b, int ldb) {
    for (int r = 0; r < nrhs; r++) {
        T* x = b + (size_t)r * ldb;
        for (int k = 0; k < n; k++) {
            const int p = ipiv[k] - 1;
            if (p != k) std::swap(x[k], x[p]);
        }
        for (int k = 0; k < n; k++) {  // L y = P b (unit diagonal)
            const T v = x[k];
            if (v == T(0)) continue;
            for (int i = k + 1; i < n; i++) x[i] -= a[i + (size_t)k * lda] * v;
        }
        for (int k = n - 1; k >= 0; k--) {  // U x = y
            x[k] /= a[k + (size_t)k * lda];
            const T v = x[k];
            if (v == T(0)) continue;
            for (int i = 0; i < k; i++) x[i] -= a[i + (size_t)k * lda] * v;
        }
    }
}

template <class T>
int potrf_lower(int n, T* a, int lda) {
    for (int j = 0; j < n; j++) {
        T d = a[j + (size_t)j * lda];
        for (int k = 0; k < j; k++) d -= a[j + (size_t)k * lda] * a[j + (size_t)k * lda];
        if (!(d > T(0))) return j + 1;
        d = std::sqrt(d);
        a[j + (size_t)j * lda] = d;
        for (int i = j + 1; i < n; i++) {
            T s = a[i + (size_t)j * lda];
            for (int k = 0; k < j; k++) s -= a[i + (size_t)k * lda] * a[j + (size_t)k * lda];
            a[i + (size_t)j * lda] = s / d;
        }
    }
    return 0;
}

template <class T>
void potrs_lower(int n, int nrhs, const T* a, int lda, T* b, int ldb) {
    for (int r = 0; r < nrhs; r++) {
        T* x = b + (size_t)r * ldb;
        for (int i = 0; i < n; i++) {
            T s = x[i];
            for (int k = 0; k < i; k++) s -= a[i + (size_t)k * lda] * x[k];
            x[i] = s / a[i + (size_t)i * lda];
        }
        for (int i = n - 1; i >= 0; i--) {
            T s = x[i];
            for (int k = i + 1; k < n; k++) s -= a[k + (size_t)i * lda] * x[k];
            x[i] = s / a[i + (size_t)i * lda];
        }
    }
}

}  // namespace

// ------------------------------------------------------------------ cuBLAS
cublasStatus_t cublasCreate(cublasHandle_t* h) {
    *h = reinterpret_cast<cublasHandle_t>(0x1);
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDestroy(cublasHandle_t) { return CUBLAS_STATUS_SUCCESS; }

template <class T>
static cublasStatus_t axpy(int n, const T* alpha, const T* x, int incx, T* y, int incy) {
    const T a = *alpha;
    for (int i = 0; i < n; i++) y[(size_t)i * incy] += a * x[(size_t)i * incx];
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDaxpy(cublasHandle_t, int n, const double* a, const double* x, int ix, double* y, int iy) {
    return axpy(n, a, x, ix, y, iy);
}
cublasStatus_t cublasSaxpy(cublasHandle_t, int n, const float* a, const float* x, int ix, float* y, int iy) {
    return axpy(n, a, x, ix, y, iy);
}
cublasStatus_t cublasDscal(cublasHandle_t, int n, const double* a, double* x, int ix) {
    for (int i = 0; i < n; i++) x[(size_t)i * ix] *= *a;
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasSscal(cublasHandle_t, int n, const float* a, float* x, int ix) {
    for (int i = 0; i < n; i++) x[(size_t)i * ix] *= *a;
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDdot(cublasHandle_t, int n, const double* x, int ix, const double* y, int iy, double* r) {
    double s = 0;
    for (int i = 0; i < n; i++) s += x[(size_t)i * ix] * y[(size_t)i * iy];
    *r = s;
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasSdot(cublasHandle_t, int n, const float* x, int ix, const float* y, int iy, float* r) {
    float s = 0;
    for (int i = 0; i < n; i++) s += x[(size_t)i * ix] * y[(size_t)i * iy];
    *r = s;
    return CUBLAS_STATUS_SUCCESS;
}
template <class T>
static cublasStatus_t getrf_batched(int n, T* const A[], int lda, int* P, int* info, int batch) {
    for (int b = 0; b < batch; b++) {
        int r = getrf<T>(n, n, A[b], lda, P + (size_t)b * n);
        if (info) info[b] = r;
    }
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDgetrfBatched(cublasHandle_t, int n, double* const A[], int lda, int* P, int* info, int batch) {
    return getrf_batched(n, A, lda, P, info, batch);
}
cublasStatus_t cublasSgetrfBatched(cublasHandle_t, int n, float* const A[], int lda, int* P, int* info, int batch) {
    return getrf_batched(n, A, lda, P, info, batch);
}
template <class T>
static cublasStatus_t getrs_batched(cublasOperation_t tr, int n, int nrhs, const T* const A[], int lda, const int* P,
                                    T* const B[], int ldb, int* info, int batch) {
    if (tr != CUBLAS_OP_N) {
        fprintf(stderr, "ref_emu: only the untransposed batched solve is provided\n");
        abort();
    }
    for (int b = 0; b < batch; b++) getrs<T>(n, nrhs, A[b], lda, P + (size_t)b * n, B[b], ldb);
    if (info) *info = 0;
    return CUBLAS_STATUS_SUCCESS;
}
cublasStatus_t cublasDgetrsBatched(cublasHandle_t, cublasOperation_t tr, int n, int nrhs, const double* const A[],
                                   int lda, const int* P, double* const B[], int ldb, int* info, int batch) {
    return getrs_batched(tr, n, nrhs, A, lda, P, B, ldb, info, batch);
}
cublasStatus_t cublasSgetrsBatched(cublasHandle_t, cublasOperation_t tr, int n, int nrhs, const float* const A[],
                                   int lda, const int* P, float* const B[], int ldb, int* info, int batch) {
    return getrs_batched(tr, n, nrhs, A, lda, P, B, ldb, info, batch);
}

// ------------------------------------------------------------------ cuSOLVER
cusolverStatus_t cusolverDnCreate(cusolverDnHandle_t* h) {
    *h = reinterpret_cast<cusolverDnHandle_t>(0x1);
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnDestroy(cusolverDnHandle_t) { return CUSOLVER_STATUS_SUCCESS; }
cusolverStatus_t cusolverDnDgetrf_bufferSize(cusolverDnHandle_t, int, int, double*, int, int* lw) {
    *lw = 1;
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnSgetrf_bufferSize(cusolverDnHandle_t, int, int, float*, int, int* lw) {
    *lw = 1;
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnDgetrf(cusolverDnHandle_t, int m, int n, double* A, int lda, double*, int* ipiv, int* info) {
    int r = getrf<double>(m, n, A, lda, ipiv);
    if (info) *info = r;
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnSgetrf(cusolverDnHandle_t, int m, int n, float* A, int lda, float*, int* ipiv, int* info) {
    int r = getrf<float>(m, n, A, lda, ipiv);
    if (info) *info = r;
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnDgetrs(cusolverDnHandle_t, cublasOperation_t tr, int n, int nrhs, const double* A, int lda,
                                  const int* ipiv, double* B, int ldb, int* info) {
    if (tr != CUBLAS_OP_N) abort();
    getrs<double>(n, nrhs, A, lda, ipiv, B, ldb);
    if (info) *info = 0;
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnSgetrs(cusolverDnHandle_t, cublasOperation_t tr, int n, int nrhs, const float* A, int lda,
                                  const int* ipiv, float* B, int ldb, int* info) {
    if (tr != CUBLAS_OP_N) abort();
    getrs<float>(n, nrhs, A, lda, ipiv, B, ldb);
    if (info) *info = 0;
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnDpotrf_bufferSize(cusolverDnHandle_t, cublasFillMode_t, int, double*, int, int* lw) {
    *lw = 1;
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnSpotrf_bufferSize(cusolverDnHandle_t, cublasFillMode_t, int, float*, int, int* lw) {
    *lw = 1;
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnDpotrf(cusolverDnHandle_t, cublasFillMode_t up, int n, double* A, int lda, double*, int,
                                  int* info) {
    if (up != CUBLAS_FILL_MODE_LOWER) abort();
    int r = potrf_lower<double>(n, A, lda);
    if (info) *info = r;
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnSpotrf(cusolverDnHandle_t, cublasFillMode_t up, int n, float* A, int lda, float*, int,
                                  int* info) {
    if (up != CUBLAS_FILL_MODE_LOWER) abort();
    int r = potrf_lower<float>(n, A, lda);
    if (info) *info = r;
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnDpotrs(cusolverDnHandle_t, cublasFillMode_t up, int n, int nrhs, const double* A, int lda,
                                  double* B, int ldb, int* info) {
    if (up != CUBLAS_FILL_MODE_LOWER) abort();
    potrs_lower<double>(n, nrhs, A, lda, B, ldb);
    if (info) *info = 0;
    return CUSOLVER_STATUS_SUCCESS;
}
cusolverStatus_t cusolverDnSpotrs(cusolverDnHandle_t, cublasFillMode_t up, int n, int nrhs, const float* A, int lda,
                                  float* B, int ldb, int* info) {
    if (up != CUBLAS_FILL_MODE_LOWER) abort();
    potrs_lower<float>(n, nrhs, A, lda, B, ldb);
    if (info) *info = 0;
    return CUSOLVER_STATUS_SUCCESS;
}
