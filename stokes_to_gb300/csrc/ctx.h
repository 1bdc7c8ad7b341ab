// Handle state shared by the 3D (solver.cu) and 2D (solver2d.cu) translation units.
#pragma once
#include <cuda_bf16.h>

#include <functional>
#include <vector>

#include "kernels.h"

namespace stg {

struct Level {
    Geom g;
    double vol = 1.0;       // vol of the free faces
    double cell_vol = 1.0;  // cell vol (reported by the descriptor adapter only)
    uint8_t* m = nullptr;
    d4* P64 = nullptr;
    float4* P32 = nullptr;
    float4 *r = nullptr, *xa = nullptr, *xb = nullptr, *rr = nullptr;
    int cur = 0;  // which of xa/xb holds the current correction
    bool lap = false;  // Laplacian-form operator valid on this level (stencil.cuh)
    __nv_bfloat16* xbf = nullptr;
    __half* P16 = nullptr;    // FP16 copy of P32 / its scale for the solver's own sweeps (set-up)
    d4 *t0 = nullptr, *t1 = nullptr;  // FP64 adapter buffers (allocated on first use)
    // general-coefficient form (general.cu; allocated on first use): per-slot vols {cell,
    // x-, y-, z-face}, the FP64 V-cycle's r, x, p, A p, and the LU-factored Vanka blocks of
    // each colour (49 doubles and 7 pivots per cell of the colour)
    d4* V64 = nullptr;
    d4 *gr = nullptr, *gx = nullptr, *gp = nullptr, *gAp = nullptr;
    double* vblk[2] = {nullptr, nullptr};
    int8_t* vpiv[2] = {nullptr, nullptr};
    float4* x() { return cur ? xb : xa; }
    float4* other() { return cur ? xa : xb; }
};

}  // namespace stg

using stg::DenseCoarse;
using stg::Level;

// A captured launch sequence (CUDA graph) and the configuration it was captured for.
struct GraphCache {
    bool enabled = true;
    cudaGraphExec_t exec = nullptr;
    long long key = -1, seen = -1, kernels = 0;
    std::vector<int> cur;          // ping-pong state of each level after the sequence
    const void* saved = nullptr;   // a pointer the sequence sets on the host (restored on replay)
    void release() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        key = -1;
    }
    ~GraphCache() { release(); }
};

// Per-kernel-class CUDA-event timing on the handle's stream.
struct Prof {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    struct Pending {
        int cls;
        size_t ev;
        double bytes;
    };
    std::vector<Pending> pend;
    long long launches[STG_PROF_NCLASS] = {};
    double ms[STG_PROF_NCLASS] = {};
    double bytes[STG_PROF_NCLASS] = {};
};

struct stg_ctx {
    int dim = 3, n = 0, L = 0;
    Prof prof;
    cudaStream_t own_st = nullptr;
    stg_opts opts{};
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    // second stream and events for host copies that overlap the set-up (stg_set_rhs)
    cudaStream_t cst = nullptr;
    cudaEvent_t ec0 = nullptr, ec1 = nullptr;
    // the set-up ran after the last penalty change, in stg_set_rhs: stg_solve skips its own
    bool setup_fresh = false;
    std::vector<stg::Level> lv;  // lv[0] coarsest ... lv[L-1] finest (reference order)
    DenseCoarse dense;
    bool closed = true, have_boundary = false, have_penalty = false, have_rhs = false, updated = false, have_solution = false;
    // lap_ok: the boundary admits the Laplacian form; general: force the masked general
    // stencil (set while an adapter works on a vector that is nonzero on fixed unknowns)
    bool lap_ok = false, general = false, reference_cycle = false;
    // gen: the boundary has non-uniform face vols or fixed cells, so the solver and the
    // adapters run the general-coefficient form (general.cu); gtmp: its finest-size scratch
    bool gen = false;
    stg::d4* gtmp[3] = {nullptr, nullptr, nullptr};
    // the coarse levels hold the solver's own penalties (flow rule of kernels.cu k_coarsen)
    // rather than the reference's sums, which the component adapters reproduce
    bool hier_flow = false;
    // a refinement step of the solve in progress ended at the basis limit short of its
    // target: the rest of the solve smooths with at least two sweeps per colour; a solve
    // that boosted makes the next solve of the handle start boosted (design loops alternate
    // forward and adjoint solves on the same, slowly changing, operator)
    bool boost = false, boost_next = false;
    bool x0_valid[2] = {false, false};  // x64 / lam64 hold a previous solution (warm start)
    bool has_x0(const stg::d4* x) const { return (x == x64 && x0_valid[0]) || (x == lam64 && x0_valid[1]); }
    int* dflag = nullptr;
    // 3D double-float copies for the FP64 residual (kernels.cu k_resid_df): x and b of the
    // solve in progress (valid while df_x / df_b name them), the low words of the finest
    // penalty (its high words are the level's P32)
    float4 *xh = nullptr, *xl = nullptr, *bh = nullptr, *bl = nullptr, *Plo = nullptr;
    // per-level scales of the FP16 penalty copies (device, level 0 coarsest) and scratch
    float* d_pscale = nullptr;
    unsigned* d_pmax = nullptr;
    const stg::d4 *df_x = nullptr, *df_b = nullptr;
    // the last residual64 call left the residual in FP32 in w (double-float iterate)
    bool r32_ok = false;
    // fine-level FP64
    stg::d4 *b64 = nullptr, *x64 = nullptr, *r64 = nullptr, *t64 = nullptr, *lam64 = nullptr;
    // Krylov (FP32)
    int m = 0;
    std::vector<float4*> V, Z;
    // FP16 copies of the basis V (3D, opts.basis16) read by the multi-dot passes, and their
    // scales (device)
    std::vector<uint2*> V16;
    float* dsc16 = nullptr;
    float4* w = nullptr;
    double *dscr = nullptr, *dh = nullptr, *dnrm = nullptr, *dy = nullptr, *dsig2 = nullptr;
    // host-order staging (cells + 3 face arrays)
    double* stage = nullptr;
    int* istage = nullptr;
    size_t ncell = 0, nface = 0;
    // design loop
    double *d_design = nullptr, *d_phys = nullptr, *d_sens = nullptr, *d_sens_design = nullptr, *d_vw = nullptr,
           *d_tmp = nullptr, *d_gauss = nullptr, *d_parts = nullptr, *d_wsum = nullptr;
    double vw_rmin = -1.0;
    const double* phys_used = nullptr;
    // fine vector length in float4 / d4 units and the per-dimension hooks of solve_core
    long long n4 = 0;
    int (*setup)(stg_t*) = nullptr;
    int (*resid64)(stg_t*, const stg::d4* b, const stg::d4* x, stg::d4* r, double* nrm2_host) = nullptr;
    int (*precond)(stg_t*, const float4* rhs, float4* out) = nullptr;
    int (*apply32)(stg_t*, const float4* x, float4* y) = nullptr;
    int (*shift32)(stg_t*, const float4* v, const float4* z, float4* out) = nullptr;  // out = v - A z
    int (*finish)(stg_t*, const stg::d4* b, stg::d4* x) = nullptr;  // optional, after the refinement loop
    struct Ctx2* c2 = nullptr;        // 2D state (dim == 2)
    struct MmaState* mma = nullptr;   // MMA optimizer state (mma.cu), created on first use
    GraphCache vgraph;                // the V-cycle below the finest level (3D) or all of it (2D)
    GraphCache vgraph_boost;          // the 3D one while `boost` raises the sweeps
    GraphCache sgraph;                // the coarsest-level set-up (probes and Gauss-Jordan inverse)
    struct NetState* net = nullptr;   // learned preconditioner (unet.cu), stg_net_init
    bool net_on = false;              // LEARNED: the network is in use in the current refinement step
};


namespace stg {
int prof_flush(stg_t* h);
int prof_begin(stg_t* h, size_t* ev);
int prof_end(stg_t* h, int cls, double bytes, size_t ev);
int solve_core(stg_t* h, const d4* b, d4* x, stg_stats* stats);
// 2D path (solver2d.cu): vectors in the reference's 8x8-blocked layout, d4 views of
// dof/4 entries. Field-order inputs are device arrays (null = zeros).
int create2d(stg_t* h);
void destroy2d(stg_t* h);
long long dof2d(const stg_t* h, int level);
int level_n2d(const stg_t* h, int level);
int set_boundary2d(stg_t* h, const double* cvol, const int* cfix, const double* fv0, const double* fv1, const int* ff0,
                   const int* ff1);
int set_penalty2d(stg_t* h, const double* cp, const double* f0, const double* f1);
int set_density2d(stg_t* h, const double* rho, const stg_alpha& law);
int field_to_vec2d(stg_t* h, const double* cell, const double* f0, const double* f1, d4* out);
int vec_to_field2d(stg_t* h, const d4* in, double* cell, double* f0, double* f1);
// out = E x; with part != nullptr, per-block partials of x.out and their count in *nb
int energy2d(stg_t* h, const d4* x, d4* out, double* part, int* nb);
int sensitivity2d(stg_t* h, const double* rho, const stg_alpha& law, const d4* x, const d4* lam, double* grad);
int apply_A2d(stg_t* h, int level, double* out, const double* in);
int apply_E2d(stg_t* h, double* out, const double* in);
int vcycle2d(stg_t* h, double* out, const double* in);
int apply_op2d(stg_t* h, int op, int level, double* out, const double* in);
int level_descr2d(stg_t* h, int level, double* vol, double* pen, uint8_t* fixed);

Level& fine(stg_t* h);
// builds the hierarchy for the adapters (reference = true) or the solves (solver.cu)
int ensure_setup(stg_t* h, bool reference);
// runs body() through a CUDA-graph cache (solver.cu)
int graphed(stg_t* h, GraphCache& G, long long key, const std::function<int()>& body, const std::function<void(bool)>& state);
bool fast(const stg_t* h, const Level& L);
// one V-cycle out = M(rhs) and y = A x on the finest level (FP32, solver.cu)
int precond3(stg_t* h, const float4* rhs, float4* out);
int apply3(stg_t* h, const float4* x, float4* y);
// z += NN(r1): the learned correction (unet.cu); net_free releases the network
int net_correct(stg_t* h, const float4* r1, float4* z);
void net_free(stg_t* h);

// General-coefficient form (general.cu): per-face vols and fixed cells
int op64v(cudaStream_t st, const Geom& g, const d4* x, const uint8_t* m, const d4* P, const d4* V, const d4* b, d4* out,
          int mode, double* part, int* nb_out);
int vol_from_field(cudaStream_t st, const Geom& g, const double* cell, const double* f0, const double* f1, const double* f2,
                   const uint8_t* m, d4* V);
int gen_setup(stg_t* h);
int gen_smooth(stg_t* h, Level& L, bool post, const d4* r_in, d4* out);
int gen_vcycle(stg_t* h);
int gen_vanka(stg_t* h, Level& L, int flag, const d4* r, d4* out);
int gen_precond(stg_t* h, const float4* rhs, float4* out);
int gen_apply32(stg_t* h, const float4* x, float4* y);
int gen_shift32(stg_t* h, const float4* v, const float4* z, float4* out);
int gen_resid64(stg_t* h, const d4* b, const d4* x, d4* r, double* nrm2_host);

// MMA design update (mma.cu) on device cell arrays; d_xout may alias d_x
int mma_update(stg_t* h, const double* d_x, const double* d_df, double frac, double coef, double lo, double hi, double movlim,
               double* d_xout, double* change);
int mma_reset(stg_t* h);
void mma_free(stg_t* h);

template <class T>
int dalloc(T** p, size_t count) {
    cudaError_t e = cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
    e = cudaMemset(*p, 0, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemset", __FILE__, __LINE__);
    return STG_OK;
}
}  // namespace stg

#define PROF(h, cls, bytes, expr)                          \
    do {                                                   \
        size_t ev_ = 0;                                    \
        STG_TRY(::stg::prof_begin((h), &ev_));             \
        STG_TRY(expr);                                     \
        STG_TRY(::stg::prof_end((h), (cls), (bytes), ev_)); \
    } while (0)
