// Host-side launchers of the grid kernels (kernels.cu, dense.cu, blas.cu, topo.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <functional>

#include "internal.cuh"

namespace stg {

// ---------------------------------------------------------------- operators (kernels.cu)
// mode: 0 out = A x, 1 out = b - A x (x == nullptr: x = 0), 2 out = E x. If part != nullptr, each block writes
// its partial sum of out.out (mode 1) or x.out (mode 2) to part[blockIdx.x] (FP64).
// lap (modes 0 and 1): Laplacian form of A (stencil.cuh) for x zero on fixed unknowns,
// rows of fixed unknowns 0. Every operator below takes the same switch; the solver sets
// it when the level satisfies the Laplacian-form conditions and its vectors are zero on
// fixed unknowns.
int op64(cudaStream_t st, const Geom& g, double vol, const d4* x, const uint8_t* m, const d4* P, const d4* b, d4* out,
         int mode, double* part, int* nblocks_out, bool lap = false);
// rr = r - A x in FP32 (x == nullptr means x = 0, so rr = r)
int resid32(cudaStream_t st, const Geom& g, float vol, const float4* r, const float4* x, const uint8_t* m, const float4* P,
            float4* rr, bool lap = false);
// y = A x in FP32
int apply32(cudaStream_t st, const Geom& g, float vol, const float4* x, const uint8_t* m, const float4* P, float4* y,
            bool lap = false);
// One colour of the box-Vanka block-Jacobi step on the residual equation, fused with the
// residual: xout = xin + SHATTER(B^-1 GATHER(r - A xin)) (sweep.cu). xin == nullptr: xin = 0.
// xc (coarse x on gc): xin is first corrected by the injected coarse value (the
// prolongation fused into the sweep; needs xin, lap and P16, else STG_E_UNSUPPORTED).
int sweep32(cudaStream_t st, const Geom& g, float vol, const float4* r, const float4* xin, float4* xout, const uint8_t* m,
            const float4* P, int flag, bool lap = false, const __half* P16 = nullptr, const float* p16_scale = nullptr,
            const float4* xc = nullptr, const Geom* gc = nullptr);
// whether the TMA-staged sweep (and with it the fused prolongation) can run here
bool sweep_tma_available();
// 1 in *timed_out when a sweep with TMA staging gave up waiting for its loads (sticky)
int sweep_status(cudaStream_t st, int* timed_out);
// rc = R (rf - A xf) with R the 8-child sum masked by the coarse mask (xf == nullptr: rc = R rf).
int restrict_resid32(cudaStream_t st, const Geom& gc, const Geom& gf, float volf, const float4* rf, const float4* xf,
                     const uint8_t* mf, const float4* Pf, const uint8_t* mc, float4* rc, bool lap = false);
// Double-float (hi + lo FP32 words) copies of FP64 vectors and the FP64 residual from them:
// hi = fl32(a), lo = fl32(a - hi) (hi may be null; part: block partials of |a|^2, 4096 at
// most, their count to *nblocks_out); r = b - A x in the Laplacian form (xh
// null: x = 0) into r (FP64) or, when r32 is non-null, rounded to FP32 into r32, with
// per-block partials of |r|^2 (FP32 per slot, double-float block sums); x = hi + lo in FP64
int split64(cudaStream_t st, long long n4, const d4* a, float4* hi, float4* lo, double* part = nullptr, int* nblocks_out = nullptr);
int resid64_df(cudaStream_t st, const Geom& g, double vol, const float4* xh, const float4* xl, const float4* bh, const float4* bl,
               const float4* Ph, const float4* Pl, const uint8_t* m, d4* r, float4* r32, double* part, int* nblocks_out);
int df_to_f64(cudaStream_t st, long long n4, const float4* hi, const float4* lo, d4* x);
// 1 in *flag (device) when x is nonzero on some fixed or absent unknown of the box, else 0
int fixed_nonzero(cudaStream_t st, const Geom& g, const d4* x, const uint8_t* m, int* flag);
// x_f = 0 on every fixed or absent unknown of the box
int zero_fixed(cudaStream_t st, const Geom& g, const uint8_t* m, d4* x);
// x_f = b_f on every fixed unknown of the box (the fixed rows of A are the identity)
int patch_fixed(cudaStream_t st, const Geom& g, const d4* b, const uint8_t* m, d4* x);
// xf += fix_f (injection of xc); linear: face values interpolated (stg_opts.prolong 1)
int prolong_add32(cudaStream_t st, const Geom& gf, const Geom& gc, const float4* xc, const uint8_t* mf, float4* xf,
                  bool linear = false);
// same with BF16-stored coarse correction
int prolong_add_bf16(cudaStream_t st, const Geom& gf, const Geom& gc, const __nv_bfloat16* xc, const uint8_t* mf, float4* xf,
                     bool linear = false);
int to_bf16(cudaStream_t st, const Geom& g, const float4* x, __nv_bfloat16* y);
// y = FP16(x / *scale) on the box slots; the per-level scales (level 0 coarsest) from the
// finest level's penalties: scale[l] = 8^(nlev-1-l) x the power of two that keeps them below 2^15
int to_f16(cudaStream_t st, const Geom& g, const float4* x, const float* scale, __half* y);
int penalty_scales(cudaStream_t st, const Geom& fine, const float4* P, int nlev, unsigned* scratch, float* scale);
// coarse descriptor from the fine one (updateSubSystem + finish); flow: velocity penalties
// by 8 x the smallest free child instead of the sum (the solver's own hierarchy)
int coarsen(cudaStream_t st, const Geom& gc, const Geom& gf, const uint8_t* mf, const d4* Pf, uint8_t* mc, d4* Pc64,
            float4* Pc32, bool flow);
// FP64 restriction / prolongation (component adapters): rc = fix_c R rf ; xf = fix_f P xc
int restrict64(cudaStream_t st, const Geom& gc, const Geom& gf, const d4* rf, const uint8_t* mc, d4* rc);
int prolong64(cudaStream_t st, const Geom& gf, const Geom& gc, const d4* xc, const uint8_t* mf, d4* xf);

// ---------------------------------------------------------------- layout (kernels.cu)
// Field-order device arrays (cell, face0..2) <-> slots. Any pointer may be null (zeros).
int field_to_slots64(cudaStream_t st, const Geom& g, const double* cell, const double* f0, const double* f1, const double* f2,
                     d4* out);
int slots_to_field64(cudaStream_t st, const Geom& g, const d4* in, double* cell, double* f0, double* f1, double* f2);
// mask = fixed flags (Field order int32, null = free) | not-present bits
int mask_from_field(cudaStream_t st, const Geom& g, const int* cell, const int* f0, const int* f1, const int* f2, uint8_t* m);
// penalty: P64 = fields zeroed on fixed; P32 = float(P64)
int penalty_from_field(cudaStream_t st, const Geom& g, const double* cell, const double* f0, const double* f1, const double* f2,
                       const uint8_t* m, d4* P64, float4* P32);
// reference blocked layout <-> slots. pad_identity: blocked padding entries copy in->out.
int blocked_to_slots64(cudaStream_t st, const Geom& g, const double* in, d4* out);
int slots_to_blocked64(cudaStream_t st, const Geom& g, const d4* in, double* out, const double* pad_src);
int mask_to_blocked(cudaStream_t st, const Geom& g, const uint8_t* m, uint8_t* out);
// descriptor vol per unknown: cell_vol on free cells, vol on free faces, 0 on fixed / absent
int vol_slots(cudaStream_t st, const Geom& g, const uint8_t* m, double cell_vol, double vol, d4* out);
// out = 1/2 x^2 per unknown
int half_square64(cudaStream_t st, long long n4, const d4* x, d4* out);

// ---------------------------------------------------------------- vectors (blas.cu)
int fill_bytes(cudaStream_t st, void* p, size_t bytes);
int f64_to_f32(cudaStream_t st, long long n4, const d4* a, double scale, float4* out);
// out = a * scale for an FP32 vector of norm 1 / scale, also writing out's FP16 copy (four
// halves per slot: the vector times a scale) and that scale to *sc_out (device)
int scale_h16(cudaStream_t st, long long n4, const float4* a, float scale, float4* out, uint2* out16, float* sc_out);
int f32_to_f64(cudaStream_t st, long long n4, const float4* a, d4* out);
// x64 += alpha * sum_j y[j] z[j]  (z FP32 vectors), y on device (nz entries); with xh / xl
// non-null also writes the double-float copy of the new x there; with x null, (xh, xl) is
// the iterate and takes the sum in double-float arithmetic; with e non-null the FP32
// value of sum_j y[j] z[j] goes to e, which may be one of z[j] for j >= axpy_last_chunk(nz)
int axpy_multi_32to64(cudaStream_t st, long long n4, const float4* const* z, const double* y, int nz, double alpha, d4* x,
                      float4* xh = nullptr, float4* xl = nullptr, float4* e = nullptr);
// first index of the last group of vectors axpy_multi_32to64 sums in one pass
int axpy_last_chunk(int nz);
// h[j] = <v_j, w> for j < nv (FP32 per-thread partials, double-float block and grid sums),
// and <w, w> into *ww when ww != nullptr

int multidot32(cudaStream_t st, long long n4, const float4* const* v, int nv, const float4* w, double* h, double* scratch,
               double* ww);
// w = v - A z (Laplacian form, slot layout of g) fused with h[q] = <V_q, w> (q < nv) and
// <w, w> into *ww (device). With V16 the first 16 dots read the vectors' FP16 copies
// instead, scaled back by 1 / sc[q] (sc on the device).
int shift_multidot32(cudaStream_t st, const Geom& g, float vol, const float4* v, const float4* z, const uint8_t* m, const float4* P,
                     long long n4, const float4* const* V, int nv, float4* w, double* h, double* scratch, double* ww,
                     const uint2* const* V16 = nullptr, const float* sc = nullptr);
// w -= sum_j h[j] v_j ; then returns ||w||^2 into nrm2 (device)
int multiaxpy32_norm(cudaStream_t st, long long n4, const float4* const* v, int nv, const double* h, float4* w, double* nrm2,
                     double* scratch);
// Classical Gram-Schmidt projection on unnormalised basis vectors in one pass:
// out = w - sum_q sig2[q] d[q] v_q (d, sig2 on the device; out may alias w); ||out||^2
// into *nrm2 and, when dots != nullptr, <v_q, out> into dots[0..nv) (device). With out16,
// also the FP16 copy of out, scaled for an out of squared norm at most *nest, the scale to
// *sc_out (nest, sc_out on the device).
int project32(cudaStream_t st, long long n4, const float4* const* v, int nv, const double* d, const double* sig2, const float4* w,
              float4* out, double* dots, double* nrm2, double* scratch, uint2* out16 = nullptr, const double* nest = nullptr,
              float* sc_out = nullptr);
// out = x / sqrt(*nrm2); with sc, the scale of x's FP16 copy follows (*sc *= sqrt(*nrm2))
int scale32(cudaStream_t st, long long n4, float4* x, const double* nrm2, float4* out, float* sc = nullptr);
// deterministic sum of nparts partials -> *out
int reduce_parts(cudaStream_t st, const double* parts, int nparts, double* out);
int dot64(cudaStream_t st, long long n4, const d4* a, const d4* b, double* out, double* scratch);

// ---------------------------------------------------------------- coarsest dense solve (dense.cu)
struct DenseCoarse {
    int nd = 0;                // number of unknowns present at the coarsest level
    int* slot_of = nullptr;    // dense index -> slot
    int* comp_of = nullptr;    // dense index -> 0 p, 1 u, 2 v, 3 w
    int* dense_of = nullptr;   // slot*4+comp -> dense index or -1
    double* A = nullptr;       // two row-major nd x 2nd buffers for Gauss-Jordan on [A | I]
    double* Ainv = nullptr;
    const double* inv = nullptr;  // the inverse: right half of the final buffer, row stride 2 nd
    int* piv = nullptr;
    int* info = nullptr;
    d4* probe = nullptr;       // probe vector and its image (slots)
    d4* image = nullptr;
    double* rd = nullptr;      // gathered right-hand side (nd)
};
int dense_init(DenseCoarse& D, const Geom& g);
void dense_free(DenseCoarse& D);
// DirectSolve3D::update: probe assembly + (closed) all-ones p-block + inversion (invert
// false: the assembly only, for a caller that captures it in a CUDA graph and then calls
// gj_invert with a cooperative launch outside the capture)
int dense_setup(cudaStream_t st, DenseCoarse& D, const Geom& g, double vol, const uint8_t* m, const d4* P64, int closed,
                bool invert = true);
// The same with per-slot face vols (general.cu op64v); extra(A, nd) may add entries to the
// assembled matrix (row-major, row stride 2 nd) before the inversion
int dense_setup_v(cudaStream_t st, DenseCoarse& D, const Geom& g, const d4* V, const uint8_t* m, const d4* P64, int closed,
                  const std::function<int(double*, int)>& extra);
// In-place Gauss-Jordan inversion of the row-major nd x 2nd [A | I] held in a (b is the
// second buffer of the same size); *inv receives the inverse (row stride 2 nd), which
// lies in whichever buffer the last step wrote. *info = first zero pivot + 1, or 0. coop:
// all steps in one cooperative launch (not capturable in a CUDA graph), else one launch
// per pivot; the two give the same inverse bit for bit.
int gj_invert(cudaStream_t st, int nd, double* a, double* b, int* info, const double** inv, bool coop = false);
// x = A^-1 r on the slots (FP32 in/out, FP64 inside)
int dense_apply32(cudaStream_t st, const DenseCoarse& D, const Geom& g, const float4* r, float4* x);
int dense_apply64(cudaStream_t st, const DenseCoarse& D, const Geom& g, const d4* r, d4* x);

// ---------------------------------------------------------------- design loop (topo.cu)
int face_penalty_from_density(cudaStream_t st, const Geom& g, const double* rho, const stg_alpha& law, const uint8_t* m,
                              d4* P64, float4* P32);
int sensitivity(cudaStream_t st, const Geom& g, const double* rho, const stg_alpha& law, const d4* x, const d4* lam,
                double* grad);
// dim 2: cells (i,j) -> i*n + j; dim 3: (i*n + j)*n + k. W: scratch of n^dim doubles
// (receives the row sums W_i).
int density_filter(cudaStream_t st, int dim, int n, double rmin, const double* in, double* out, int transpose, double* W);
int oc_volume(cudaStream_t st, int ncell, const double* x, const double* dc, const double* vw, double lam, double move,
              double lo, double hi, double* xnew, double* parts, int* nparts);
// The whole OC update (bracket, bisection, x_new) in one cooperative launch; parts: two
// buffers of up to 1216 block partials; lambda_out: one device double.
int oc_update_device(cudaStream_t st, int ncell, const double* x, const double* dc, const double* vw, double frac,
                     double move, double lo, double hi, double* xnew, double* parts, double* lambda_out);
int density_noise(cudaStream_t st, int dim, int n, uint64_t seed, const double* w, int R, double* out, double* tmp);

}  // namespace stg
