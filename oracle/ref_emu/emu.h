// Host-side stand-in for the CUDA language and runtime, used to run the reference's own
// CUDA solver code on the CPU. TEST INFRASTRUCTURE ONLY: it serves oracle/ref_emu, which
// turns the reference's kernels and host classes into golden vectors that pin the
// oracle; the product library never sees it.
//
// Execution model: a launch runs its blocks one after another; inside a block every
// thread is a fiber (ucontext) and __syncthreads() switches to the next fiber, so a
// barrier completes once every live thread of the block has reached it. Block-shared
// variables are function-local statics (one block runs at a time). A kernel whose first
// thread finishes without meeting a barrier is run thread by thread as plain calls; a
// barrier met later in that mode is a fatal error. Atomics are plain read-modify-writes
// (one host thread). Device memory is host memory.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__
#define __shared__ static
#define __constant__
#define __launch_bounds__(...)

struct uint3 {
    unsigned x, y, z;
};
struct dim3 {
    unsigned x, y, z;
    dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

extern uint3 threadIdx;
extern uint3 blockIdx;
extern dim3 blockDim;
extern dim3 gridDim;
static const int warpSize = 32;

void __syncthreads();
inline void __threadfence() {}

inline double atomicAdd(double* p, double v) {
    double o = *p;
    *p = o + v;
    return o;
}
inline float atomicAdd(float* p, float v) {
    float o = *p;
    *p = o + v;
    return o;
}
inline int atomicAdd(int* p, int v) {
    int o = *p;
    *p = o + v;
    return o;
}
inline unsigned atomicAdd(unsigned* p, unsigned v) {
    unsigned o = *p;
    *p = o + v;
    return o;
}

// device math overloads that CUDA provides at global scope
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline double min(double a, double b) { return fmin(a, b); }
inline double max(double a, double b) { return fmax(a, b); }
inline float min(float a, float b) { return fminf(a, b); }
inline float max(float a, float b) { return fmaxf(a, b); }

namespace emu {
struct Cfg {
    dim3 g, b;
    Cfg(dim3 g_, dim3 b_, size_t = 0, void* = nullptr) : g(g_), b(b_) {}
};
// runs body once per thread of every block of the launch (see the execution model above)
void launch(const Cfg& c, const std::function<void()>& body);
}  // namespace emu

// ------------------------------------------------------------------ runtime API subset
typedef enum cudaError {
    cudaSuccess = 0,
    cudaErrorInvalidValue = 1,
    cudaErrorMemoryAllocation = 2,
} cudaError_t;
typedef enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
} cudaMemcpyKind;
typedef struct CUstream_st* cudaStream_t;

cudaError_t cudaMalloc(void** p, size_t bytes);
template <class T>
inline cudaError_t cudaMalloc(T** p, size_t bytes) {
    return cudaMalloc(reinterpret_cast<void**>(p), bytes);
}
cudaError_t cudaFree(void* p);
cudaError_t cudaMemcpy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind);
cudaError_t cudaMemset(void* p, int v, size_t bytes);
cudaError_t cudaDeviceSynchronize();
cudaError_t cudaGetLastError();
cudaError_t cudaPeekAtLastError();
cudaError_t cudaDeviceReset();
const char* cudaGetErrorName(cudaError_t e);
const char* cudaGetErrorString(cudaError_t e);

// ------------------------------------------------------------------ cuBLAS subset
typedef struct cublasContext* cublasHandle_t;
typedef enum { CUBLAS_STATUS_SUCCESS = 0, CUBLAS_STATUS_INVALID_VALUE = 7 } cublasStatus_t;
typedef enum { CUBLAS_OP_N = 0, CUBLAS_OP_T = 1, CUBLAS_OP_C = 2 } cublasOperation_t;
typedef enum { CUBLAS_FILL_MODE_LOWER = 0, CUBLAS_FILL_MODE_UPPER = 1 } cublasFillMode_t;

cublasStatus_t cublasCreate(cublasHandle_t* h);
cublasStatus_t cublasDestroy(cublasHandle_t h);
cublasStatus_t cublasDaxpy(cublasHandle_t, int n, const double* alpha, const double* x, int incx, double* y, int incy);
cublasStatus_t cublasSaxpy(cublasHandle_t, int n, const float* alpha, const float* x, int incx, float* y, int incy);
cublasStatus_t cublasDscal(cublasHandle_t, int n, const double* alpha, double* x, int incx);
cublasStatus_t cublasSscal(cublasHandle_t, int n, const float* alpha, float* x, int incx);
cublasStatus_t cublasDdot(cublasHandle_t, int n, const double* x, int incx, const double* y, int incy, double* r);
cublasStatus_t cublasSdot(cublasHandle_t, int n, const float* x, int incx, const float* y, int incy, float* r);
cublasStatus_t cublasDgetrfBatched(cublasHandle_t, int n, double* const A[], int lda, int* P, int* info, int batch);
cublasStatus_t cublasSgetrfBatched(cublasHandle_t, int n, float* const A[], int lda, int* P, int* info, int batch);
cublasStatus_t cublasDgetrsBatched(cublasHandle_t, cublasOperation_t trans, int n, int nrhs, const double* const A[],
                                   int lda, const int* P, double* const B[], int ldb, int* info, int batch);
cublasStatus_t cublasSgetrsBatched(cublasHandle_t, cublasOperation_t trans, int n, int nrhs, const float* const A[],
                                   int lda, const int* P, float* const B[], int ldb, int* info, int batch);

// ------------------------------------------------------------------ cuSOLVER dense subset
typedef struct cusolverDnContext* cusolverDnHandle_t;
typedef enum { CUSOLVER_STATUS_SUCCESS = 0 } cusolverStatus_t;

cusolverStatus_t cusolverDnCreate(cusolverDnHandle_t* h);
cusolverStatus_t cusolverDnDestroy(cusolverDnHandle_t h);
cusolverStatus_t cusolverDnDgetrf_bufferSize(cusolverDnHandle_t, int m, int n, double* A, int lda, int* lwork);
cusolverStatus_t cusolverDnSgetrf_bufferSize(cusolverDnHandle_t, int m, int n, float* A, int lda, int* lwork);
cusolverStatus_t cusolverDnDgetrf(cusolverDnHandle_t, int m, int n, double* A, int lda, double* work, int* ipiv,
                                  int* info);
cusolverStatus_t cusolverDnSgetrf(cusolverDnHandle_t, int m, int n, float* A, int lda, float* work, int* ipiv,
                                  int* info);
cusolverStatus_t cusolverDnDgetrs(cusolverDnHandle_t, cublasOperation_t trans, int n, int nrhs, const double* A,
                                  int lda, const int* ipiv, double* B, int ldb, int* info);
cusolverStatus_t cusolverDnSgetrs(cusolverDnHandle_t, cublasOperation_t trans, int n, int nrhs, const float* A,
                                  int lda, const int* ipiv, float* B, int ldb, int* info);
cusolverStatus_t cusolverDnDpotrf_bufferSize(cusolverDnHandle_t, cublasFillMode_t, int n, double* A, int lda,
                                             int* lwork);
cusolverStatus_t cusolverDnDpotrf(cusolverDnHandle_t, cublasFillMode_t, int n, double* A, int lda, double* work,
                                  int lwork, int* info);
cusolverStatus_t cusolverDnDpotrs(cusolverDnHandle_t, cublasFillMode_t, int n, int nrhs, const double* A, int lda,
                                  double* B, int ldb, int* info);
cusolverStatus_t cusolverDnSpotrf_bufferSize(cusolverDnHandle_t, cublasFillMode_t, int n, float* A, int lda,
                                             int* lwork);
cusolverStatus_t cusolverDnSpotrf(cusolverDnHandle_t, cublasFillMode_t, int n, float* A, int lda, float* work,
                                  int lwork, int* info);
cusolverStatus_t cusolverDnSpotrs(cusolverDnHandle_t, cublasFillMode_t, int n, int nrhs, const float* A, int lda,
                                  float* B, int ldb, int* info);
