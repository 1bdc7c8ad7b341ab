// Host orchestration of libstokes_gb300 and its C ABI (include/stokes_gb300.h).
//
// 3D solve = FluidSteadyState3D::solve (stoke/FluidSteadyState3D.cpp:152-170) re-designed
// for one GB300: the coarse re-discretisation, the smoother blocks and the coarsest
// inverse are rebuilt on the device; the reference's host GMRES with the V-cycle as
// left preconditioner (common_cpx/GMRES.cpp:20-110) becomes a device-resident FP64
// defect-correction loop whose correction equations are solved by right-preconditioned
// FGMRES in FP32 with the same V-cycle (common_cpx/MultigridSolve.cpp:73-114) as
// preconditioner. Every vector stays in HBM; the host only sees the Hessenberg scalars.
// The 2D path (FluidSteadyState, stoke/FluidSteadyState.cpp) lives in solver2d.cu and
// plugs its set-up, residual, preconditioner and operator into the same driver.
#include <cuda_bf16.h>

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <functional>
#include <vector>

#include "ctx.h"

namespace stg {

static thread_local char g_err[512] = "";
static std::atomic<long long> g_launches{0};

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void add_launches(long long k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    const char* base = strrchr(file, '/');
    set_error("%s:%d %s: %s", base ? base + 1 : file, line, what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? STG_E_NOMEM : STG_E_CUDA;
}

}  // namespace stg

using namespace stg;

namespace stg {

Level& fine(stg_t* h) { return h->lv[h->L - 1]; }

// the Laplacian-form kernels apply: the level admits them and the vectors in flight are
// zero on fixed unknowns (always inside solve_core; adapters check their input)
bool fast(const stg_t* h, const Level& L) { return L.lap && !h->general; }

int prof_flush(stg_t* h) {
    Prof& P = h->prof;
    if (P.pend.empty()) return STG_OK;
    STG_CK(cudaEventSynchronize(P.pool[P.used - 1]));
    for (auto& q : P.pend) {
        float ms = 0;
        STG_CK(cudaEventElapsedTime(&ms, P.pool[q.ev], P.pool[q.ev + 1]));
        P.ms[q.cls] += ms;
        P.bytes[q.cls] += q.bytes;
        P.launches[q.cls]++;
    }
    P.pend.clear();
    P.used = 0;
    return STG_OK;
}

int prof_begin(stg_t* h, size_t* ev) {
    Prof& P = h->prof;
    if (!P.on) return STG_OK;
    if (P.used + 2 > P.pool.size()) STG_TRY(prof_flush(h));
    while (P.pool.size() < P.used + 2) {
        cudaEvent_t e;
        STG_CK(cudaEventCreate(&e));
        P.pool.push_back(e);
    }
    *ev = P.used;
    STG_CK(cudaEventRecord(P.pool[P.used++], h->st));
    return STG_OK;
}

int prof_end(stg_t* h, int cls, double bytes, size_t ev) {
    Prof& P = h->prof;
    if (!P.on) return STG_OK;
    STG_CK(cudaEventRecord(P.pool[P.used++], h->st));
    P.pend.push_back({cls, ev, bytes});
    if (P.used >= 8192) STG_TRY(prof_flush(h));
    return STG_OK;
}


int level_count(int n) {
    int low = n & -n;
    int l = (int)std::lround(std::log2((double)low)) - 1;
    return l < 1 ? 1 : l;
}

double* stage_cell(stg_t* h) { return h->stage; }
double* stage_face(stg_t* h, int d) { return h->stage + h->ncell + (size_t)d * h->nface; }

int upload_fields(stg_t* h, const double* cell, const double* const* faces, const double** dc, const double** df) {
    if (cell) STG_CK(cudaMemcpyAsync(stage_cell(h), cell, sizeof(double) * h->ncell, cudaMemcpyHostToDevice, h->st));
    *dc = cell ? stage_cell(h) : nullptr;
    for (int d = 0; d < h->dim; d++) {
        const double* f = faces ? faces[d] : nullptr;
        if (f) STG_CK(cudaMemcpyAsync(stage_face(h, d), f, sizeof(double) * h->nface, cudaMemcpyHostToDevice, h->st));
        df[d] = f ? stage_face(h, d) : nullptr;
    }
    return STG_OK;
}

int download_fields(stg_t* h, const d4* src, double* cell, double* const* faces) {
    if (h->dim == 2)
        STG_TRY(vec_to_field2d(h, src, stage_cell(h), stage_face(h, 0), stage_face(h, 1)));
    else
        STG_TRY(slots_to_field64(h->st, fine(h).g, src, stage_cell(h), stage_face(h, 0), stage_face(h, 1), stage_face(h, 2)));
    if (cell) STG_CK(cudaMemcpyAsync(cell, stage_cell(h), sizeof(double) * h->ncell, cudaMemcpyDeviceToHost, h->st));
    for (int d = 0; d < h->dim; d++)
        if (faces && faces[d])
            STG_CK(cudaMemcpyAsync(faces[d], stage_face(h, d), sizeof(double) * h->nface, cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

// Field-order device arrays -> the fine-level FP64 vector of either dimension
int fields_to_vec(stg_t* h, const double* dc, const double* const* df, d4* out) {
    if (h->dim == 2) return field_to_vec2d(h, dc, df[0], df[1], out);
    return field_to_slots64(h->st, fine(h).g, dc, df[0], df[1], df[2], out);
}

// out = E x on the fine level; part != nullptr also gives the per-block partials of x.out
int energy_op(stg_t* h, const d4* x, d4* out, double* part, int* nb) {
    if (h->dim == 2) return energy2d(h, x, out, part, nb);
    Level& F = fine(h);
    if (h->gen) return op64v(h->st, F.g, x, F.m, F.P64, F.V64, nullptr, out, 2, part, nb);
    return op64(h->st, F.g, F.vol, x, F.m, F.P64, nullptr, out, 2, part, nb);
}

// ---------------------------------------------------------------- hierarchy set-up
// FluidSteadyState3D::solve set-up (stoke/FluidSteadyState3D.cpp:155-156): coarse
// descriptors (updateSubSystem) and the coarsest inverse (DirectSolve3D::update). The
// smoother blocks need no set-up: the kernels form them from the level coefficients.
int update(stg_t* h) {
    if (!h->have_boundary || !h->have_penalty) {
        set_error("boundary and penalty must be set before the solver set-up");
        return STG_E_INVALID;
    }
    for (int i = h->L - 2; i >= 0; i--) {
        Level &c = h->lv[i], &f = h->lv[i + 1];
        PROF(h, 8, 0.0, coarsen(h->st, c.g, f.g, f.m, f.P64, c.m, c.P64, c.P32, h->hier_flow));
        c.vol = 4.0 * f.vol;
        c.cell_vol = 8.0 * f.cell_vol;
    }
    // coarse boundary faces have fixed children, so the Laplacian form carries down
    for (auto& L : h->lv) L.lap = h->lap_ok;
    if (h->gen) {
        PROF(h, 8, 0.0, gen_setup(h));
        h->updated = true;
        return STG_OK;
    }
    // FP16 copies of the penalties for the solver's own sweeps, each level divided by a scale
    // that keeps it in FP16's range (11 significant bits: the V-cycle count is the FP32 one)
    PROF(h, 8, 0.0, penalty_scales(h->st, fine(h).g, fine(h).P32, h->L, h->d_pmax, h->d_pscale));
    for (int i = 0; i < h->L; i++) PROF(h, 8, 0.0, to_f16(h->st, h->lv[i].g, h->lv[i].P32, h->d_pscale + i, h->lv[i].P16));
    // low words of the finest penalty for the double-float residual (P32 holds the high)
    PROF(h, 8, 0.0, split64(h->st, fine(h).g.nslot, fine(h).P64, nullptr, h->Plo));
    // the coarsest matrix's assembly (27 small launches) reads and writes fixed buffers:
    // replayed as a CUDA graph; its Gauss-Jordan inversion is one cooperative launch
    GraphCache& G = h->sgraph;
    PROF(h, 8, 0.0,
         graphed(h, G, h->closed ? 2 : 1,
                 [&] {
                     return dense_setup(h->st, h->dense, h->lv[0].g, h->lv[0].vol, h->lv[0].m, h->lv[0].P64, h->closed ? 1 : 0,
                                        false);
                 },
                 [](bool) {}));
    PROF(h, 8, 0.0, gj_invert(h->st, h->dense.nd, h->dense.A, h->dense.Ainv, h->dense.info, &h->dense.inv, true));
    h->updated = true;
    return STG_OK;
}

// Builds the hierarchy when it is missing or was built for the other kind of caller: the
// component adapters (reference = true) reproduce the reference's coarse penalties, the
// solves use the flow rule.
int ensure_setup(stg_t* h, bool reference) {
    const bool flow = !reference;
    if (h->updated && h->hier_flow == flow) return STG_OK;
    h->hier_flow = flow;
    return h->setup(h);
}

// ---------------------------------------------------------------- V-cycle (FP32)
// Smoother of StokeLike::GenerateJacobiPreconditioner(grid, A, 2) (stoke/StokeLike.cu:345-372):
// DescentSmoother({red, black}, {2, 2}) before the coarse correction and {black, red} after
// (common_cpx/DescentSmoother.cu:31-47), written in correction form x <- x + P_c(r - A x).
int sweep(stg_t* h, Level& L, const float4* r, int flag, bool first, Level* C = nullptr) {
    float vol = (float)L.vol;
    // profile class 1: sweeps of the finest level; 10: of the coarser levels
    const int cls = &L == &fine(h) ? 1 : 10;
    // the adapters keep the FP32 penalty (the reference smoother to FP32 rounding); the
    // solver's sweeps stage the level's FP16 copy with its scale (sweep.cu SmemT)
    const __half* P16 = h->reference_cycle ? nullptr : L.P16;
    const float* psc = h->d_pscale + (&L - h->lv.data());
    if (first) {
        // x = 0: the residual is r itself
        PROF(h, cls, 41.0 * L.g.box(), sweep32(h->st, L.g, vol, r, nullptr, L.x(), L.m, L.P32, flag, fast(h, L), P16, psc));
        return STG_OK;
    }
    if (C) {  // with the coarse correction injected as x is staged: 2 B a slot more
        PROF(h, cls, 59.0 * L.g.box(),
             sweep32(h->st, L.g, vol, r, L.x(), L.other(), L.m, L.P32, flag, fast(h, L), P16, psc, C->x(), &C->g));
        L.cur ^= 1;
        return STG_OK;
    }
    PROF(h, cls, 57.0 * L.g.box(), sweep32(h->st, L.g, vol, r, L.x(), L.other(), L.m, L.P32, flag, fast(h, L), P16, psc));
    L.cur ^= 1;
    return STG_OK;
}

// The prolongation (injection) can ride on the first post-smoothing sweep: FP32 coarse
// correction, the solver's own uniform-form sweeps (TMA, FP16 penalty) with x present.
bool fuse_prolong(const stg_t* h, const Level& F) {
    return !h->reference_cycle && h->opts.method != STG_METHOD_MIXED && h->opts.prolong != 1 && fast(h, F) && F.P16 &&
           sweep_tma_available();
}

// Sweeps per colour: the reference's 2 for the adapters, else the solver option, raised to
// 2 for the rest of a solve whose refinement step stalled.
int sweeps_per_colour(const stg_t* h) {
    if (h->reference_cycle) return 2;
    const int s = std::max(1, std::min(4, h->opts.smooth_sweeps));
    return h->boost ? std::max(s, 2) : s;
}

// C: the coarse level whose correction the first sweep injects (fuse_prolong)
int smooth(stg_t* h, Level& L, const float4* r, bool post, bool x_is_zero, Level* C = nullptr) {
    const int per = sweeps_per_colour(h);
    int s = 0;
    for (int c = 0; c < 2; c++) {
        const int flag = post ? 1 - c : c;
        for (int q = 0; q < per; q++, s++) STG_TRY(sweep(h, L, r, flag, s == 0 && x_is_zero, s == 0 ? C : nullptr));
    }
    return STG_OK;
}

// MultigridSolve::Vcycle (common_cpx/MultigridSolve.cpp:73-106) from a zero guess on levels
// top .. 0: level i < L - 1 takes its right-hand side from its own r; the finest level's is
// `rhs`. The result is left in lv[top].x().
int vcycle_levels(stg_t* h, int top, const float4* rhs) {
    const bool mixed = h->opts.method == STG_METHOD_MIXED;
    const bool lin = h->opts.prolong == 1 && !h->reference_cycle;
    const int L = h->L;
    for (int i = top; i >= 1; i--) {
        Level& F = h->lv[i];
        const float4* r = (i == L - 1) ? rhs : F.r;
        F.cur = 0;
        STG_TRY(smooth(h, F, r, false, true));
        Level& C = h->lv[i - 1];
        PROF(h, 2, 49.0 * F.g.box() + 17.0 * C.g.box(), restrict_resid32(h->st, C.g, F.g, (float)F.vol, r, F.x(), F.m, F.P32, C.m, C.r, fast(h, F)));
    }
    Level& C0 = h->lv[0];
    C0.cur = 0;
    PROF(h, 7, 0.0, dense_apply32(h->st, h->dense, C0.g, L == 1 ? rhs : C0.r, C0.x()));
    for (int i = 1; i <= top; i++) {
        Level& F = h->lv[i];
        Level& C = h->lv[i - 1];
        const float4* r = (i == L - 1) ? rhs : F.r;
        if (fuse_prolong(h, F)) {
            STG_TRY(smooth(h, F, r, true, false, &C));
            continue;
        }
        if (mixed) {
            PROF(h, 3, 24.0 * C.g.box(), to_bf16(h->st, C.g, C.x(), C.xbf));
            PROF(h, 3, 8.0 * C.g.box() + 33.0 * F.g.box(), prolong_add_bf16(h->st, F.g, C.g, C.xbf, F.m, F.x(), lin));
        } else {
            PROF(h, 3, 16.0 * C.g.box() + 33.0 * F.g.box(), prolong_add32(h->st, F.g, C.g, C.x(), F.m, F.x(), lin));
        }
        STG_TRY(smooth(h, F, r, true, false));
    }
    return STG_OK;
}

// Runs body() through the graph cache G: a launch sequence that touches only fixed
// buffers is captured into a CUDA graph on its second call with the same configuration
// `key` (the first runs normally, so one-time set-up such as kernel attributes happens
// outside the capture) and replayed on later calls. state(true) records the host-side state
// the sequence leaves, state(false) restores it after a replay. Off while the per-kernel
// profiler is on.
int graphed(stg_t* h, GraphCache& G, long long key, const std::function<int()>& body, const std::function<void(bool)>& state) {
    if (h->prof.on || !G.enabled) return body();
    if (G.exec && G.key == key) {
        STG_CK(cudaGraphLaunch(G.exec, h->st));
        add_launches(G.kernels);
        state(false);
        return STG_OK;
    }
    if (G.seen != key) {
        G.seen = key;
        return body();
    }
    G.release();
    cudaGraph_t graph = nullptr;
    STG_CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
    const long long l0 = stg_kernel_launches();
    const int rc = body();
    const cudaError_t e = cudaStreamEndCapture(h->st, &graph);
    if (rc != STG_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    G.kernels = stg_kernel_launches() - l0;  // counted during the capture: they stand for the first replay
    const cudaError_t e2 = cudaGraphInstantiate(&G.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e2 != cudaSuccess) {
        G.exec = nullptr;
        return cuda_fail(e2, "cudaGraphInstantiate", __FILE__, __LINE__);
    }
    G.key = key;
    state(true);
    STG_CK(cudaGraphLaunch(G.exec, h->st));
    return STG_OK;
}

// The levels below the finest touch only their own buffers, so their part of the V-cycle is
// the same launch sequence on every call and runs as a replayed CUDA graph.
int coarse_cycle(stg_t* h) {
    const int top = h->L - 2;
    const int per = sweeps_per_colour(h);
    // the coarsest inverse lives in one of two buffers (fixed per handle): part of the key
    const long long key = (long long)per | ((long long)(h->opts.method == STG_METHOD_MIXED) << 3) |
                          ((long long)fast(h, h->lv[top]) << 4) | ((long long)(h->dense.inv == h->dense.Ainv) << 5) |
                          ((long long)h->L << 6) | ((long long)h->reference_cycle << 12) |  // adapters: FP32 sweeps
                          ((long long)(h->opts.prolong == 1) << 13);
    GraphCache& G = h->boost && !h->reference_cycle ? h->vgraph_boost : h->vgraph;
    return graphed(h, G, key, [&] { return vcycle_levels(h, top, nullptr); },
                   [&](bool save) {
                       if (save) {
                           G.cur.assign(top + 1, 0);
                           for (int i = 0; i <= top; i++) G.cur[i] = h->lv[i].cur;
                       } else {
                           for (int i = 0; i <= top; i++) h->lv[i].cur = G.cur[i];
                       }
                   });
}

// MultigridSolve::Vcycle (common_cpx/MultigridSolve.cpp:73-106) from a zero guess; the
// finest right-hand side is `rhs`, the result is left in fine(h).x().
int vcycle(stg_t* h, const float4* rhs) {
    const int L = h->L;
    if (L == 1) return vcycle_levels(h, 0, rhs);
    const bool mixed = h->opts.method == STG_METHOD_MIXED;
    Level& F = h->lv[L - 1];
    Level& C = h->lv[L - 2];
    F.cur = 0;
    STG_TRY(smooth(h, F, rhs, false, true));
    PROF(h, 2, 49.0 * F.g.box() + 17.0 * C.g.box(), restrict_resid32(h->st, C.g, F.g, (float)F.vol, rhs, F.x(), F.m, F.P32, C.m, C.r, fast(h, F)));
    STG_TRY(coarse_cycle(h));
    if (fuse_prolong(h, F)) return smooth(h, F, rhs, true, false, &C);
    const bool lin = h->opts.prolong == 1 && !h->reference_cycle;
    if (mixed) {
        PROF(h, 3, 24.0 * C.g.box(), to_bf16(h->st, C.g, C.x(), C.xbf));
        PROF(h, 3, 8.0 * C.g.box() + 33.0 * F.g.box(), prolong_add_bf16(h->st, F.g, C.g, C.xbf, F.m, F.x(), lin));
    } else {
        PROF(h, 3, 16.0 * C.g.box() + 33.0 * F.g.box(), prolong_add32(h->st, F.g, C.g, C.x(), F.m, F.x(), lin));
    }
    return smooth(h, F, rhs, true, false);
}

// ---------------------------------------------------------------- FP64 refinement + FGMRES
int residual64(stg_t* h, const d4* b, const d4* x, d4* r, double* nrm2_host) {
    Level& F = fine(h);
    int nb = 0;
    h->r32_ok = false;
    if ((!x || x == h->df_x) && b == h->df_b && fast(h, F)) {
        // the solve's iterate is the double-float pair (xh, xl): the residual, rounded to
        // FP32 (the Krylov basis is built from it), goes to h->w
        PROF(h, 5, (x ? 113.0 : 49.0) * F.g.box(),
             resid64_df(h->st, F.g, F.vol, x ? h->xh : nullptr, x ? h->xl : nullptr, h->bh, h->bl, F.P32, h->Plo, F.m, nullptr, h->w,
                        h->d_parts, &nb));
        h->r32_ok = true;
    } else {
        PROF(h, 5, (x ? 129.0 : 65.0) * F.g.box(), op64(h->st, F.g, F.vol, x, F.m, F.P64, b, r, 1, h->d_parts, &nb, fast(h, F)));
    }
    STG_TRY(reduce_parts(h->st, h->d_parts, nb, h->dnrm));
    STG_CK(cudaMemcpyAsync(nrm2_host, h->dnrm, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

// 3D hooks of solve_core
int precond3(stg_t* h, const float4* rhs, float4* out) {
    Level& F = fine(h);
    // the V-cycle leaves its result in the finest level's second buffer: point it at out
    float4* keep = F.xb;
    F.xb = out;
    int vrc = vcycle(h, rhs);
    float4* res = F.x();
    F.xb = keep;
    STG_TRY(vrc);
    if (res != out) STG_CK(cudaMemcpyAsync(out, res, sizeof(float4) * F.g.nslot, cudaMemcpyDeviceToDevice, h->st));
    return STG_OK;
}

// STG_METHOD_LEARNED: out = S(M(rhs) + NN(rhs - A M(rhs))) while the network is in use,
// S one post-smoothing pass of the finest level on A out = rhs (it removes the rough part
// of the network's error, which A would amplify in the residual). h->w is free here: the
// Arnoldi step overwrites it with A out next.
int precond_learned(stg_t* h, const float4* rhs, float4* out) {
    STG_TRY(precond3(h, rhs, out));
    if (!h->net_on) return STG_OK;
    Level& F = fine(h);
    PROF(h, 4, 49.0 * F.g.box(), resid32(h->st, F.g, (float)F.vol, rhs, out, F.m, F.P32, h->w, fast(h, F)));
    PROF(h, 11, 0.0, net_correct(h, h->w, out));
    // smooth in place: the level's ping-pong buffers point at out and h->w; an even
    // number of sweeps leaves the result in out
    float4 *ka = F.xa, *kb = F.xb;
    const int kc = F.cur;
    F.xa = out;
    F.xb = h->w;
    F.cur = 0;
    const int rc = smooth(h, F, rhs, true, false);
    F.xa = ka;
    F.xb = kb;
    F.cur = kc;
    return rc;
}

int shift3(stg_t* h, const float4* v, const float4* z, float4* out) {
    Level& F = fine(h);
    PROF(h, 4, 65.0 * F.g.box(), resid32(h->st, F.g, (float)F.vol, v, z, F.m, F.P32, out, fast(h, F)));
    return STG_OK;
}

int apply3(stg_t* h, const float4* x, float4* y) {
    Level& F = fine(h);
    PROF(h, 4, 49.0 * F.g.box(), apply32(h->st, F.g, (float)F.vol, x, F.m, F.P32, y, fast(h, F)));
    return STG_OK;
}

// The Laplacian-form residual leaves the fixed rows at 0 and x at 0 there; the fixed
// rows of A are the identity, so the fixed part of the solution is b_f exactly.
int finish3(stg_t* h, const d4* b, d4* x) {
    Level& F = fine(h);
    if (fast(h, F)) STG_TRY(patch_fixed(h->st, F.g, b, F.m, x));
    return STG_OK;
}

int solve_core(stg_t* h, const d4* b, d4* x, stg_stats* stats) {
    const long long n4 = h->n4;
    stg_stats S{};
    if (!h->updated || !h->hier_flow) {
        auto t0 = std::chrono::steady_clock::now();
        STG_TRY(ensure_setup(h, false));
        STG_CK(cudaStreamSynchronize(h->st));
        S.setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    STG_CK(cudaEventRecord(h->e0, h->st));
    // 3D Laplacian form: the iterate is kept as a double-float pair (xh, xl) during the solve
    // (FP32 arithmetic only: GB300's FP64 pipe is far slower than HBM for per-element work)
    // and formed in FP64 once at the end; b is split the same way for the FP64 residual
    const bool df = h->dim == 3 && fast(h, fine(h));
    // the fused operator + multi-dot pass (3D uniform form) reads the basis's FP16 copies
    const bool h16 = df && !h->V16.empty();
    // zero initial guess as the reference, or the previous solution of this equation
    if (h->opts.warm_start && h->has_x0(x)) {
        if (df) STG_TRY(zero_fixed(h->st, fine(h).g, fine(h).m, x));
    } else if (!df) {
        STG_CK(cudaMemsetAsync(x, 0, sizeof(d4) * n4, h->st));
    }
    if (h->opts.method == STG_METHOD_LEARNED && !h->net) {
        set_error("STG_METHOD_LEARNED needs a network (stg_net_init, then stg_net_train or stg_net_set_params)");
        return STG_E_INVALID;
    }
    if (h->opts.warm_start == 2 && (!h->net || h->dim != 3)) {
        set_error("the learned warm start (warm_start 2) needs a 3D handle with a network");
        return STG_E_INVALID;
    }
    h->net_on = h->opts.method == STG_METHOD_LEARNED;
    // a zero start makes the first residual b itself (fixed rows cleared in the Laplacian form)
    bool x_zero = !(h->opts.warm_start && h->has_x0(x));
    h->df_x = h->df_b = nullptr;
    double bn2 = 0;
    if (df) {
        if (x_zero) {
            STG_CK(cudaMemsetAsync(h->xh, 0, sizeof(float4) * n4, h->st));
            STG_CK(cudaMemsetAsync(h->xl, 0, sizeof(float4) * n4, h->st));
        } else {
            PROF(h, 6, 64.0 * n4, split64(h->st, n4, x, h->xh, h->xl));
        }
        int nbp = 0;  // ||b||^2 from the same pass
        PROF(h, 6, 64.0 * n4, split64(h->st, n4, b, h->bh, h->bl, h->d_parts, &nbp));
        STG_TRY(reduce_parts(h->st, h->d_parts, nbp, h->dnrm));
        h->df_x = x;
        h->df_b = b;
    } else {
        STG_TRY(dot64(h->st, n4, b, b, h->dnrm, h->dscr));
    }
    STG_CK(cudaMemcpyAsync(&bn2, h->dnrm, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    const double bn = std::sqrt(bn2);
    const int m = h->m;
    // Augmented restarts (as LGMRES): the corrections of the last refinement steps that ran
    // out of basis are kept in the last basis slots Z[m-1], Z[m-2], ... and take the place
    // of the last Krylov steps of the following refinement steps. Restarted FGMRES discards
    // the few slow directions it had found on every restart; the stored corrections carry
    // them over (the iteration-5 design of the 256^3 loop at fraction 0.15: 600 V-cycles
    // without, 270 with four). The slots must lie in the first group the update sums.
    const int naug = std::max(0, std::min({4, m / 2, m - axpy_last_chunk(m)}));
    int have_aug = 0, aug_next = 0;  // filled slots Z[m-have_aug .. m-1]; next to overwrite
    bool stalled_any = false;  // a refinement step of this solve ran out of basis
    struct BoostGuard {
        stg_t* h;
        const bool& stalled;
        ~BoostGuard() {
            h->boost_next = stalled;
            h->boost = false;
        }
    } boost_guard{h, stalled_any};
    h->boost = h->boost_next && h->dim == 3 && !h->net_on;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m), hcol(m + 2), sig(m + 1);
    double rel = 0, rn = 0;
    int status = STG_E_NOT_CONVERGED;
    for (int outer = 0; outer <= h->opts.max_outer; outer++) {
        double rn2 = 0;
        STG_TRY(h->resid64(h, b, (outer == 0 && x_zero && h->dim == 3) ? nullptr : x, h->r64, &rn2));
        rn = std::sqrt(rn2);
        if (outer == 0 && !x_zero && rn > bn) {
            // the previous solution is further from this one than zero is (the design moved
            // a lot, e.g. when it first turns into a channel): start from zero instead
            if (h->opts.verbose) fprintf(stderr, "[stg] warm start rejected (||b-Ax0||/||b|| = %.3e)\n", bn > 0 ? rn / bn : 0.0);
            x_zero = true;
            if (!df) STG_CK(cudaMemsetAsync(x, 0, sizeof(d4) * n4, h->st));
            if (df) {
                STG_CK(cudaMemsetAsync(h->xh, 0, sizeof(float4) * n4, h->st));
                STG_CK(cudaMemsetAsync(h->xl, 0, sizeof(float4) * n4, h->st));
            }
            STG_TRY(h->resid64(h, b, h->dim == 3 ? nullptr : x, h->r64, &rn2));
            rn = std::sqrt(rn2);
        }
        rel = bn > 0 ? rn / bn : 0.0;
        if (!std::isfinite(rn)) {
            status = STG_E_NONFINITE;
            set_error("non-finite FP64 residual at refinement step %d", outer);
            break;
        }
        if (h->opts.verbose) fprintf(stderr, "[stg] outer %d  ||b-Ax||/||b|| = %.3e\n", outer, rel);
        if (rel <= h->opts.tol || rn == 0.0) {
            status = STG_OK;
            break;
        }
        if (outer == h->opts.max_outer) break;
        S.outer_iters++;
        // v0 = r / ||r|| in FP32
        if (h->r32_ok && h16)
            PROF(h, 6, 40.0 * n4, scale_h16(h->st, n4, h->w, (float)(1.0 / rn), h->V[0], h->V16[0], h->dsc16));
        else if (h->r32_ok)
            PROF(h, 6, 32.0 * n4, scale32(h->st, n4, h->w, h->dnrm, h->V[0]));
        else
            PROF(h, 6, 48.0 * n4, f64_to_f32(h->st, n4, h->r64, 1.0 / rn, h->V[0]));
        double beta = 1.0;
        // ask this step for what the target still needs, within [inner_tol / 10, inner_tol]
        const double itol = std::min(h->opts.inner_tol, std::max(0.3 * h->opts.tol / rel, 0.1 * h->opts.inner_tol));
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int k = 0;
        // The basis is kept unnormalised: v_q = sig_q V_q with sig_q = 1/||V_q|| held on the
        // host (and sig_q^2 on the device), z_q = sig_q Z_q with Z_q = M V_q. Arnoldi step:
        // pass 1 d1 = V^T w; pass 2 V_{j+1} = w - sum sig^2 d1 V together with
        // d2 = V^T V_{j+1}; pass 3 (classical Gram-Schmidt's second sweep, only when the
        // first cancelled nearly all of w: ||V_{j+1}|| < 0.1 ||w||) V_{j+1} -= sum sig^2 d2 V.
        // The looser trigger than the usual 0.7 costs orthogonality of order 1e-6 in FP32,
        // far below the 1e-4 an inner solve is asked for; the FP64 refinement decides.
        sig[0] = 1.0;
        const double one = 1.0;
        STG_CK(cudaMemcpyAsync(h->dsig2, &one, sizeof(double), cudaMemcpyHostToDevice, h->st));
        double prev_est = beta;
        // Learned warm start (warm_start 2): the first refinement step of a warm-started solve
        // is one FGMRES step whose preconditioner is the learned correction, i.e. the
        // previous solution plus the step along the network-corrected V-cycle of its
        // residual that minimises the new residual (never worse than the plain warm start)
        const bool predict = h->opts.warm_start == 2 && outer == 0 && !x_zero;
        const int msteps = predict ? 1 : m;
        for (int j = 0; j < msteps; j++) {
            const bool aug_step = j >= m - have_aug;  // Z[j] holds a stored correction
            if (predict) {
                S.learned_iters++;
                const bool keep = h->net_on;
                h->net_on = true;
                const int prc = precond_learned(h, h->V[j], h->Z[j]);
                h->net_on = keep;
                STG_TRY(prc);
            } else if (!aug_step) {
                if (h->net_on) S.learned_iters++;
                STG_TRY(h->precond(h, h->V[j], h->Z[j]));
            }
            // Arnoldi on the shifted operator A M - I, written as w = V_j - A Z_j: same Krylov
            // space, and a good preconditioner (A M near I) no longer leaves w dominated by
            // V_j, whose removal cancelled most of w and forced the second projection pass
            if (h->dim == 3 && fast(h, fine(h))) {
                // one pass: the operator and the first multi-dot (w is not re-read)
                Level& F = fine(h);
                const int nh = h16 ? std::min(j + 1, 16) : 0;  // dots read from the FP16 copies
                PROF(h, 6, (65.0 + 16.0 * (j + 1) - 8.0 * nh) * F.g.box(),
                     shift_multidot32(h->st, F.g, (float)F.vol, h->V[j], h->Z[j], F.m, F.P32, n4, h->V.data(), j + 1, h->w, h->dh,
                                      h->dscr, h->dnrm + 1, h16 ? h->V16.data() : nullptr, h->dsc16));
            } else {
                STG_TRY(h->shift32(h, h->V[j], h->Z[j], h->w));
                PROF(h, 6, 16.0 * (j + 2) * n4, multidot32(h->st, n4, h->V.data(), j + 1, h->w, h->dh, h->dscr, h->dnrm + 1));
            }
            // the new vector's FP16 copy is scaled for a norm up to ||w|| (the projection only
            // shortens w); a second projection rewrites it for its own input's norm
            PROF(h, 6, (16.0 * (j + 3) + (h16 ? 8.0 : 0.0)) * n4,
                 project32(h->st, n4, h->V.data(), j + 1, h->dh, h->dsig2, h->w, h->V[j + 1], h->dh + m + 2, h->dnrm, h->dscr,
                           h16 ? h->V16[j + 1] : nullptr, h->dnrm + 1, h->dsc16 + j + 1));
            std::vector<double> h1(j + 1), h2(j + 1, 0.0);
            double nrm[2] = {0, 0};
            STG_CK(cudaMemcpyAsync(h1.data(), h->dh, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, h->st));
            STG_CK(cudaMemcpyAsync(h2.data(), h->dh + m + 2, sizeof(double) * (j + 1), cudaMemcpyDeviceToHost, h->st));
            STG_CK(cudaMemcpyAsync(nrm, h->dnrm, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
            STG_CK(cudaStreamSynchronize(h->st));
            double nw2 = nrm[0];
            if (nrm[0] < 0.01 * nrm[1]) {
                PROF(h, 6, (16.0 * (j + 3) + (h16 ? 8.0 : 0.0)) * n4,
                     project32(h->st, n4, h->V.data(), j + 1, h->dh + m + 2, h->dsig2, h->V[j + 1], h->V[j + 1], nullptr, h->dnrm,
                               h->dscr, h16 ? h->V16[j + 1] : nullptr, h->dnrm, h->dsc16 + j + 1));
                STG_CK(cudaMemcpyAsync(&nw2, h->dnrm, sizeof(double), cudaMemcpyDeviceToHost, h->st));
                STG_CK(cudaStreamSynchronize(h->st));
            } else {
                std::fill(h2.begin(), h2.end(), 0.0);
            }
            S.inner_iters++;
            // A z_j = v_j - sum_q sig_q sig_j d_q v_q - (sig_j / sig_{j+1}) v_{j+1}
            const double hn = sig[j] * std::sqrt(nw2);
            for (int q = 0; q <= j; q++) hcol[q] = (q == j ? 1.0 : 0.0) - sig[q] * sig[j] * (h1[q] + h2[q]);
            hcol[j + 1] = -hn;
            if (!std::isfinite(hn)) {
                status = STG_E_NONFINITE;
                set_error("non-finite Arnoldi norm");
                break;
            }
            if (nw2 > 1e8 || (nw2 > 0 && nw2 < 1e-8)) {
                // the unnormalised basis drifts in scale by the gain of A M each step (large
                // for a weak preconditioner on high-contrast designs): renormalise before FP32
                // over- or underflows
                PROF(h, 6, 32.0 * n4, scale32(h->st, n4, h->V[j + 1], h->dnrm, h->V[j + 1], h16 ? h->dsc16 + j + 1 : nullptr));
                sig[j + 1] = 1.0;
                const double one1 = 1.0;
                STG_CK(cudaMemcpyAsync(h->dsig2 + j + 1, &one1, sizeof(double), cudaMemcpyHostToDevice, h->st));
            } else if (nw2 > 0) {
                sig[j + 1] = 1.0 / std::sqrt(nw2);
                const double s2 = 1.0 / nw2;
                STG_CK(cudaMemcpyAsync(h->dsig2 + j + 1, &s2, sizeof(double), cudaMemcpyHostToDevice, h->st));
            }
            // Givens rotations on the new Hessenberg column
            for (int q = 0; q < j; q++) {
                double a = hcol[q], c = hcol[q + 1];
                hcol[q] = cs[q] * a + sn[q] * c;
                hcol[q + 1] = -sn[q] * a + cs[q] * c;
            }
            double a = hcol[j], c = hcol[j + 1];
            double den = std::hypot(a, c);
            cs[j] = den > 0 ? a / den : 1.0;
            sn[j] = den > 0 ? c / den : 0.0;
            hcol[j] = den;
            hcol[j + 1] = 0.0;
            for (int q = 0; q <= j; q++) H[q + (size_t)j * (m + 1)] = hcol[q];
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            k = j + 1;
            double est = std::fabs(g[j + 1]);
            if (h->opts.verbose > 1) fprintf(stderr, "[stg]   inner %d  est %.3e\n", j, est);
            // a learned step that cut the estimate by less than 20% ends the network's use in
            // this solve (FGMRES is flexible, so the basis built so far stays valid). The
            // first step of a refinement step is not assessed: its reduction depends on how
            // the right-hand side lies (a boundary-driven b gives about 2% with plain
            // multigrid too).
            if (h->net_on && j > 0 && !aug_step && est > 0.8 * prev_est) {
                h->net_on = false;
                S.fallbacks++;
            }
            prev_est = est;
            if (est <= itol * beta || hn == 0.0) break;
        }
        if (status == STG_E_NONFINITE) break;
        for (int q = k - 1; q >= 0; q--) {
            double s = g[q];
            for (int c = q + 1; c < k; c++) s -= H[q + (size_t)c * (m + 1)] * y[c];
            double d = H[q + (size_t)q * (m + 1)];
            y[q] = d != 0 ? s / d : 0.0;
        }
        for (int q = 0; q < k; q++) y[q] *= sig[q];  // z_q = sig_q Z_q
        STG_CK(cudaMemcpyAsync(h->dy, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, h->st));
        // the step used the whole basis short of its target
        const bool stalled = k == m && std::fabs(g[k]) > itol * beta;
        float4* keep = nullptr;
        if (stalled && naug > 0) {
            // the oldest stored correction (or a free slot) takes this step's correction for
            // a unit residual, so that A Z_j is of the order of the basis vector it is taken from
            keep = h->Z[m - 1 - aug_next];
            aug_next = (aug_next + 1) % naug;
            have_aug = std::min(naug, have_aug + 1);
        }
        PROF(h, 6, (16.0 * k + 64.0 + (keep ? 16.0 : 0.0)) * n4,
             axpy_multi_32to64(h->st, n4, h->Z.data(), h->dy, k, rn, df ? nullptr : x, df ? h->xh : nullptr, df ? h->xl : nullptr,
                               keep));
        // a stalled step means the V-cycle is too weak for this design (high-contrast
        // optimised densities): the rest of the solve smooths twice per colour (about 1.5x
        // the V-cycle's cost for 1.5-2x fewer V-cycles there)
        if (h->dim == 3 && stalled) h->boost = stalled_any = true;
    }
    if (df) PROF(h, 6, 64.0 * n4, df_to_f64(h->st, n4, h->xh, h->xl, x));  // the iterate in FP64
    h->df_x = h->df_b = nullptr;  // finish() changes x; adapters must not see the copies
    if (h->finish) STG_TRY(h->finish(h, b, x));
    int sweep_timeout = 0;
    STG_TRY(sweep_status(h->st, &sweep_timeout));
    if (sweep_timeout) {
        set_error("smoother sweep: a staging wait timed out");
        return STG_E_CUDA;
    }
    STG_CK(cudaEventRecord(h->e1, h->st));
    STG_CK(cudaEventSynchronize(h->e1));
    float ms = 0;
    STG_CK(cudaEventElapsedTime(&ms, h->e0, h->e1));
    S.solve_ms = ms;
    STG_TRY(prof_flush(h));
    S.rel_residual = rel;
    S.abs_residual = rn;
    S.status = status;
    if (stats) *stats = S;
    if (status == STG_E_NOT_CONVERGED) set_error("tolerance %.1e not reached (%.3e after %d steps)", h->opts.tol, rel, S.outer_iters);
    return status;
}

// Adapters take any vector; the Laplacian form needs zero fixed entries, so a vector
// that has nonzero fixed entries runs the general stencil for this call.
struct PathGuard {
    stg_t* h;
    ~PathGuard() {
        h->general = false;
        h->reference_cycle = false;
    }
};

int choose_path(stg_t* h, const Level& L, const d4* x) {
    h->general = false;
    h->reference_cycle = true;  // adapters reproduce the reference's V-cycle and smoother
    if (!L.lap) return STG_OK;
    int nz = 0;
    STG_TRY(fixed_nonzero(h->st, L.g, x, L.m, h->dflag));
    STG_CK(cudaMemcpyAsync(&nz, h->dflag, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    h->general = nz != 0;
    return STG_OK;
}

int ensure_adapter(Level& L) {
    if (!L.t0) STG_TRY(dalloc(&L.t0, L.g.nslot));
    if (!L.t1) STG_TRY(dalloc(&L.t1, L.g.nslot));
    return STG_OK;
}

int check_handle(const stg_t* h) {
    if (!h) {
        set_error("null handle");
        return STG_E_INVALID;
    }
    return STG_OK;
}

}  // namespace stg

// ====================================================================== C ABI
extern "C" {

void stg_default_opts(stg_opts* o) {
    if (!o) return;
    o->method = STG_METHOD_PLAIN;
    o->tol = 1e-8;
    o->max_outer = 20;
    o->inner_max = 30;
    o->inner_tol = 1e-4;
    o->verbose = 0;
    o->smooth_sweeps = 1;
    o->warm_start = 0;
    o->prolong = 0;
    o->basis16 = 1;
}

const char* stg_last_error(void) { return g_err; }

int stg_set_stream(stg_t* h, void* cuda_stream) {
    STG_TRY(check_handle(h));
    STG_CK(cudaStreamSynchronize(h->st));
    h->st = cuda_stream ? (cudaStream_t)cuda_stream : h->own_st;
    return STG_OK;
}

int64_t stg_kernel_launches(void) { return g_launches.load(); }

int stg_profile(stg_t* h, int enable) {
    STG_TRY(check_handle(h));
    STG_TRY(prof_flush(h));
    Prof& P = h->prof;
    P.on = enable != 0;
    for (int c = 0; c < STG_PROF_NCLASS; c++) {
        P.launches[c] = 0;
        P.ms[c] = 0;
        P.bytes[c] = 0;
    }
    return STG_OK;
}

int stg_profile_read(stg_t* h, int cls, int64_t* launches, double* ms, double* bytes) {
    STG_TRY(check_handle(h));
    if (cls < 0 || cls >= STG_PROF_NCLASS) {
        set_error("bad profile class %d", cls);
        return STG_E_INVALID;
    }
    STG_TRY(prof_flush(h));
    if (launches) *launches = h->prof.launches[cls];
    if (ms) *ms = h->prof.ms[cls];
    if (bytes) *bytes = h->prof.bytes[cls];
    return STG_OK;
}

const char* stg_profile_name(int cls) {
    static const char* names[STG_PROF_NCLASS] = {"resid32", "sweep32", "restrict32", "prolong32", "apply32", "resid64",
                                                 "krylov",  "coarse",  "setup",      "other",     "sweep32_coarse", "net"};
    return (cls >= 0 && cls < STG_PROF_NCLASS) ? names[cls] : "";
}

const char* stg_version(void) { return "stokes_gb300 0.1 (sm_103a)"; }

int stg_create(int dim, int n, const stg_opts* opts, stg_t** out) {
    if (!out) {
        set_error("null output handle");
        return STG_E_INVALID;
    }
    *out = nullptr;
    if (dim != 2 && dim != 3) {
        set_error("dim %d: must be 2 or 3", dim);
        return STG_E_INVALID;
    }
    if (dim == 3 && (n < 4 || n % 4 != 0)) {
        set_error("N = %d must be a positive multiple of 4", n);
        return STG_E_INVALID;
    }
    if (dim == 3 && n > 1024) {
        set_error("N = %d exceeds the 32-bit slot indexing limit of 1024", n);
        return STG_E_UNSUPPORTED;
    }
    if (dim == 2 && (n < 8 || n % 8 != 0)) {
        set_error("N = %d must be a positive multiple of 8 (8x8-blocked 2D layout)", n);
        return STG_E_INVALID;
    }
    if (dim == 2 && n > 16384) {
        set_error("N = %d exceeds the 32-bit 2D indexing limit of 16384", n);
        return STG_E_UNSUPPORTED;
    }
    stg_t* h = new stg_t();
    h->dim = dim;
    h->n = n;
    if (opts)
        h->opts = *opts;
    else
        stg_default_opts(&h->opts);
    if (h->opts.inner_max < 1) h->opts.inner_max = 1;
    if (h->opts.smooth_sweeps < 1) h->opts.smooth_sweeps = 1;  // unset: the default
    // 2D vectors are small: keep at least the reference GMRES's 60-vector basis there (high-
    // contrast 2D designs need long Krylov runs per refinement step)
    h->m = dim == 2 ? std::max(h->opts.inner_max, 60) : h->opts.inner_max;
    h->L = dim == 3 ? level_count(n) : 0;
    int rc = STG_OK;
    auto fail = [&](int r) {
        stg_destroy(h);
        return r;
    };
    if (cudaStreamCreateWithFlags(&h->own_st, cudaStreamNonBlocking) != cudaSuccess) {
        set_error("cudaStreamCreate failed");
        delete h;
        return STG_E_CUDA;
    }
    h->st = h->own_st;
    cudaEventCreate(&h->e0);
    cudaEventCreate(&h->e1);
    if (cudaStreamCreateWithFlags(&h->cst, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ec0, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ec1, cudaEventDisableTiming) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "create", __FILE__, __LINE__));
    if (dim == 2 && (rc = create2d(h))) return fail(rc);
    h->lv.resize(dim == 3 ? h->L : 0);
    for (int i = (int)h->lv.size() - 1, nn = n; i >= 0; i--, nn /= 2) {
        Level& L = h->lv[i];
        L.g = Geom::make(nn);
        size_t ns = L.g.nslot;
        if ((rc = dalloc(&L.m, ns)) || (rc = dalloc(&L.P64, ns)) || (rc = dalloc(&L.P32, ns)) || (rc = dalloc(&L.r, ns)) ||
            (rc = dalloc(&L.xa, ns)) || (rc = dalloc(&L.xb, ns)) || (rc = dalloc(&L.rr, ns)) ||
            (rc = dalloc(&L.xbf, 4 * ns)) || (rc = dalloc(&L.P16, 4 * ns)))
            return fail(rc);
        // halo and absent unknowns fixed; the box is rewritten by set_boundary / coarsen
        if ((rc = mask_from_field(h->st, L.g, nullptr, nullptr, nullptr, nullptr, L.m))) return fail(rc);
    }
    long long nparts = 0;
    if (dim == 2 && h->opts.method == STG_METHOD_LEARNED) {
        set_error("STG_METHOD_LEARNED: 3D handles only");
        return fail(STG_E_INVALID);
    }
    if (dim == 3) {
        if ((rc = dense_init(h->dense, h->lv[0].g))) return fail(rc);
        Level& F = fine(h);
        h->n4 = (long long)F.g.nslot;
        h->setup = update;
        h->resid64 = residual64;
        h->precond = h->opts.method == STG_METHOD_LEARNED ? precond_learned : precond3;
        h->apply32 = apply3;
        h->shift32 = shift3;
        h->finish = finish3;
        h->ncell = (size_t)n * n * n;
        h->nface = (size_t)n * n * (n + 1);
        nparts = grid_for(F.g.box(), 256);
    } else {
        nparts = grid_for(4 * h->n4, 256);
    }
    const size_t ns = (size_t)h->n4;
    if ((rc = dalloc(&h->b64, ns)) || (rc = dalloc(&h->x64, ns)) || (rc = dalloc(&h->r64, ns)) || (rc = dalloc(&h->t64, ns)) ||
        (rc = dalloc(&h->lam64, ns)) || (rc = dalloc(&h->w, ns)) ||
        (dim == 3 && ((rc = dalloc(&h->xh, ns)) || (rc = dalloc(&h->xl, ns)) || (rc = dalloc(&h->bh, ns)) || (rc = dalloc(&h->bl, ns)) ||
                      (rc = dalloc(&h->Plo, ns)) || (rc = dalloc(&h->d_pscale, (size_t)h->L)) || (rc = dalloc(&h->d_pmax, 1)))))
        return fail(rc);
    h->V.assign(h->m + 1, nullptr);
    h->Z.assign(h->m, nullptr);
    for (auto& p : h->V)
        if ((rc = dalloc(&p, ns))) return fail(rc);
    for (auto& p : h->Z)
        if ((rc = dalloc(&p, ns))) return fail(rc);
    if (dim == 3 && h->opts.basis16) {
        // the FP16 copies only speed up the multi-dot: without room for them the handle
        // runs on the FP32 basis alone
        h->V16.assign(h->m + 1, nullptr);
        bool ok = dalloc(&h->dsc16, (size_t)h->m + 1) == STG_OK;
        for (auto& p : h->V16) ok = ok && dalloc(&p, ns) == STG_OK;
        if (!ok) {
            for (auto p : h->V16) cudaFree(p);
            cudaFree(h->dsc16);
            h->V16.clear();
            h->dsc16 = nullptr;
            cudaGetLastError();
            set_error("%s", "");
        }
    }
    if ((rc = dalloc(&h->dscr, 1216 * 18)) || (rc = dalloc(&h->dh, 2 * (h->m + 2))) || (rc = dalloc(&h->dnrm, 8)) ||
        (rc = dalloc(&h->dsig2, h->m + 2)) ||
        (rc = dalloc(&h->dy, h->m + 1)) || (rc = dalloc(&h->d_parts, (size_t)nparts + 1216)) || (rc = dalloc(&h->dflag, 1)))
        return fail(rc);
    if ((rc = dalloc(&h->stage, h->ncell + 3 * h->nface)) || (rc = dalloc(&h->istage, h->ncell + 3 * h->nface))) return fail(rc);
    if ((rc = dalloc(&h->d_design, h->ncell)) || (rc = dalloc(&h->d_phys, h->ncell)) || (rc = dalloc(&h->d_sens, h->ncell)) ||
        (rc = dalloc(&h->d_sens_design, h->ncell)) || (rc = dalloc(&h->d_vw, h->ncell)) || (rc = dalloc(&h->d_tmp, h->ncell)) ||
        (rc = dalloc(&h->d_wsum, h->ncell)) ||
        (rc = dalloc(&h->d_gauss, 512)))
        return fail(rc);
    if (cudaStreamSynchronize(h->st) != cudaSuccess) return fail(cuda_fail(cudaGetLastError(), "create", __FILE__, __LINE__));
    *out = h;
    return STG_OK;
}

int stg_destroy(stg_t* h) {
    if (!h) return STG_OK;
    if (h->st) cudaStreamSynchronize(h->st);
    destroy2d(h);
    mma_free(h);
    net_free(h);
    for (auto& L : h->lv) {
        cudaFree(L.m);
        cudaFree(L.P64);
        cudaFree(L.P32);
        cudaFree(L.r);
        cudaFree(L.xa);
        cudaFree(L.xb);
        cudaFree(L.rr);
        cudaFree(L.xbf);
        cudaFree(L.P16);
        cudaFree(L.t0);
        cudaFree(L.t1);
        cudaFree(L.V64);
        for (d4* p : {L.gr, L.gx, L.gp, L.gAp}) cudaFree(p);
        for (int c = 0; c < 2; c++) {
            cudaFree(L.vblk[c]);
            cudaFree(L.vpiv[c]);
        }
    }
    for (d4* p : h->gtmp) cudaFree(p);
    dense_free(h->dense);
    for (d4* p : {h->b64, h->x64, h->r64, h->t64, h->lam64}) cudaFree(p);
    cudaFree(h->w);
    for (float4* p : {h->xh, h->xl, h->bh, h->bl, h->Plo}) cudaFree(p);
    cudaFree(h->d_pscale);
    cudaFree(h->d_pmax);
    for (auto p : h->V) cudaFree(p);
    for (auto p : h->V16) cudaFree(p);
    cudaFree(h->dsc16);
    for (auto p : h->Z) cudaFree(p);
    for (double* p : {h->dscr, h->dh, h->dnrm, h->dy, h->dsig2, h->stage, h->d_design, h->d_phys, h->d_sens, h->d_sens_design, h->d_vw,
                      h->d_tmp, h->d_gauss, h->d_parts, h->d_wsum})
        cudaFree(p);
    cudaFree(h->istage);
    cudaFree(h->dflag);
    if (h->e0) cudaEventDestroy(h->e0);
    if (h->e1) cudaEventDestroy(h->e1);
    for (auto e : h->prof.pool) cudaEventDestroy(e);
    if (h->own_st) cudaStreamDestroy(h->own_st);
    if (h->cst) cudaStreamDestroy(h->cst);
    if (h->ec0) cudaEventDestroy(h->ec0);
    if (h->ec1) cudaEventDestroy(h->ec1);
    delete h;
    return STG_OK;
}

int stg_set_method(stg_t* h, int method) {
    STG_TRY(check_handle(h));
    if (method < STG_METHOD_PLAIN || method > STG_METHOD_LEARNED || (method == STG_METHOD_LEARNED && h->dim != 3)) {
        set_error("stg_set_method: method %d not available for dim %d", method, h->dim);
        return STG_E_INVALID;
    }
    if (h->gen && method == STG_METHOD_LEARNED) {
        set_error("STG_METHOD_LEARNED needs uniform face vols and free cells");
        return STG_E_UNSUPPORTED;
    }
    h->opts.method = method;
    if (h->dim == 3 && !h->gen) h->precond = method == STG_METHOD_LEARNED ? precond_learned : precond3;
    return STG_OK;
}

int stg_levels(const stg_t* h) { return h ? h->L : 0; }
int stg_level_n(const stg_t* h, int level) {
    if (!h || level < 0 || level >= h->L) return 0;
    return h->dim == 2 ? level_n2d(h, level) : h->lv[level].g.n;
}
int64_t stg_level_dof(const stg_t* h, int level) {
    if (!h || level < 0 || level >= h->L) return 0;
    if (h->dim == 2) return dof2d(h, level);
    Blocked B{h->lv[level].g.n};
    return B.size();
}

int stg_set_boundary(stg_t* h, const double* cell_vol, const int32_t* cell_fixed, const double* const* face_vol,
                     const int32_t* const* face_fixed, int closed) {
    STG_TRY(check_handle(h));
    if (!face_vol || !face_fixed) {
        set_error("face_vol and face_fixed are required");
        return STG_E_INVALID;
    }
    if (h->dim == 2) {
        // the 2D kernels read every coefficient from the descriptor: any vol, fixed cells allowed
        for (int d = 0; d < 2; d++)
            if (!face_vol[d] || !face_fixed[d]) {
                set_error("face arrays of axis %d missing", d);
                return STG_E_INVALID;
            }
        const double* dc = nullptr;
        const double* df[3] = {nullptr, nullptr, nullptr};
        STG_TRY(upload_fields(h, cell_vol, face_vol, &dc, df));
        int* ist = h->istage;
        if (cell_fixed) STG_CK(cudaMemcpyAsync(ist, cell_fixed, sizeof(int) * h->ncell, cudaMemcpyHostToDevice, h->st));
        for (int d = 0; d < 2; d++)
            STG_CK(cudaMemcpyAsync(ist + h->ncell + d * h->nface, face_fixed[d], sizeof(int) * h->nface, cudaMemcpyHostToDevice,
                                   h->st));
        STG_TRY(set_boundary2d(h, dc, cell_fixed ? ist : nullptr, df[0], df[1], ist + h->ncell, ist + h->ncell + h->nface));
        h->closed = closed != 0;
        h->have_boundary = true;
        h->updated = false;
        STG_CK(cudaStreamSynchronize(h->st));
        return STG_OK;
    }
    const int n = h->n;
    // the uniform-coefficient form needs one vol value on the free faces and no fixed cell;
    // anything else runs the general-coefficient form (general.cu)
    double v = NAN;
    bool gen = false;
    for (int d = 0; d < 3; d++) {
        if (!face_vol[d] || !face_fixed[d]) {
            set_error("face arrays of axis %d missing", d);
            return STG_E_INVALID;
        }
        for (size_t q = 0; q < h->nface && !gen; q++) {
            if (face_fixed[d][q]) continue;
            if (std::isnan(v)) v = face_vol[d][q];
            if (face_vol[d][q] != v) gen = true;
        }
    }
    if (cell_fixed)
        for (size_t q = 0; q < h->ncell && !gen; q++)
            if (cell_fixed[q]) gen = true;
    if (gen && h->opts.method == STG_METHOD_LEARNED) {
        set_error("STG_METHOD_LEARNED needs uniform face vols and free cells");
        return STG_E_UNSUPPORTED;
    }
    // Laplacian form: every face on the domain boundary fixed (Field order, N+1 along d)
    bool bnd_fixed = true;
    for (int d = 0; d < 3 && bnd_fixed; d++)
        for (int a = 0; a <= n && bnd_fixed; a++)
            for (int b = 0; b < n && bnd_fixed; b++)
                for (int c = 0; c < n && bnd_fixed; c++) {
                    if (a != 0 && a != n) continue;
                    int ijk[3];
                    ijk[d] = a;
                    ijk[(d + 1) % 3] = b;
                    ijk[(d + 2) % 3] = c;
                    const size_t q = ((size_t)ijk[0] * (n + (d == 1)) + ijk[1]) * (n + (d == 2)) + ijk[2];
                    if (!face_fixed[d][q]) bnd_fixed = false;
                }
    h->lap_ok = bnd_fixed && !gen;
    double cv = cell_vol ? cell_vol[0] : 1.0;
    Level& F = fine(h);
    F.vol = std::isnan(v) ? 0.0 : v;
    F.cell_vol = cv;
    int* ist = h->istage;
    const int* fi[3];
    for (int d = 0; d < 3; d++) {
        STG_CK(cudaMemcpyAsync(ist + h->ncell + d * h->nface, face_fixed[d], sizeof(int) * h->nface, cudaMemcpyHostToDevice,
                               h->st));
        fi[d] = ist + h->ncell + d * h->nface;
    }
    const int* fc = nullptr;
    if (gen && cell_fixed) {
        STG_CK(cudaMemcpyAsync(ist, cell_fixed, sizeof(int) * h->ncell, cudaMemcpyHostToDevice, h->st));
        fc = ist;
    }
    STG_TRY(mask_from_field(h->st, F.g, fc, fi[0], fi[1], fi[2], F.m));
    h->gen = gen;
    if (gen) {
        // per-slot vols (0 on fixed unknowns, as the reference's finish() leaves them)
        if (!F.V64 && dalloc(&F.V64, F.g.nslot)) return STG_E_CUDA;
        const double* dc = nullptr;
        const double* df[3] = {nullptr, nullptr, nullptr};
        STG_TRY(upload_fields(h, cell_vol, face_vol, &dc, df));
        STG_TRY(vol_from_field(h->st, F.g, dc, df[0], df[1], df[2], F.m, F.V64));
        h->resid64 = gen_resid64;
        h->precond = gen_precond;
        h->apply32 = gen_apply32;
        h->shift32 = gen_shift32;
    } else {
        h->resid64 = residual64;
        h->precond = h->opts.method == STG_METHOD_LEARNED ? precond_learned : precond3;
        h->apply32 = apply3;
        h->shift32 = shift3;
    }
    h->closed = closed != 0;
    h->have_boundary = true;
    h->updated = false;
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_set_penalty(stg_t* h, const double* cell_penalty, const double* const* face_penalty) {
    STG_TRY(check_handle(h));
    if (!h->have_boundary) {
        set_error("stg_set_boundary must come first");
        return STG_E_INVALID;
    }
    const double* dc = nullptr;
    const double* df[3] = {nullptr, nullptr, nullptr};
    STG_TRY(upload_fields(h, cell_penalty, face_penalty, &dc, df));
    if (h->dim == 2) {
        STG_TRY(set_penalty2d(h, dc, df[0], df[1]));
    } else {
        Level& F = fine(h);
        STG_TRY(penalty_from_field(h->st, F.g, dc, df[0], df[1], df[2], F.m, F.P64, F.P32));
    }
    h->have_penalty = true;
    h->updated = false;
    h->phys_used = nullptr;
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_set_rhs(stg_t* h, const double* cell_b, const double* const* face_b) {
    STG_TRY(check_handle(h));
    const double* dc = nullptr;
    const double* df[3] = {nullptr, nullptr, nullptr};
    // A pending 3D set-up (the penalty changed since the last one) reads only the penalty
    // and the boundary: it runs on the handle's stream while b is copied on the copy
    // stream, and the next stg_solve uses it instead of running its own.
    const bool overlap = h->dim == 3 && h->have_boundary && h->have_penalty && (!h->updated || !h->hier_flow);
    if (overlap) {
        STG_CK(cudaEventRecord(h->ec0, h->st));  // earlier work on the staging buffer first
        STG_CK(cudaStreamWaitEvent(h->cst, h->ec0, 0));
        cudaStream_t keep = h->st;
        h->st = h->cst;
        const int urc = upload_fields(h, cell_b, face_b, &dc, df);
        h->st = keep;
        STG_TRY(urc);
        STG_CK(cudaEventRecord(h->ec1, h->cst));
        const int src = ensure_setup(h, false);
        // the handle's stream takes the copy over in every case, so no later call finds
        // the staging buffer still being written
        STG_CK(cudaStreamWaitEvent(h->st, h->ec1, 0));
        if (src != STG_OK) {
            cudaStreamSynchronize(h->cst);
            return src;
        }
        h->setup_fresh = true;
    } else {
        STG_TRY(upload_fields(h, cell_b, face_b, &dc, df));
    }
    STG_TRY(fields_to_vec(h, dc, df, h->b64));
    h->have_rhs = true;
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_solve(stg_t* h, double* p_out, double* const* vel_out, stg_stats* stats) {
    STG_TRY(check_handle(h));
    if (!h->have_rhs) {
        set_error("stg_set_rhs must come first");
        return STG_E_INVALID;
    }
    // the reference re-runs the set-up on every solve; one that stg_set_rhs ran after the
    // last penalty change (overlapping the copy of b) counts as this solve's
    if (!h->setup_fresh) h->updated = false;
    h->setup_fresh = false;
    int rc = solve_core(h, h->b64, h->x64, stats);
    if (rc != STG_OK && rc != STG_E_NOT_CONVERGED) return rc;
    h->have_solution = true;
    h->x0_valid[0] = true;
    if (p_out || vel_out) STG_TRY(download_fields(h, h->x64, p_out, vel_out));
    return rc;
}

int stg_get_solution(stg_t* h, double* p_out, double* const* vel_out) {
    STG_TRY(check_handle(h));
    if (!h->have_solution) {
        set_error("no solution yet");
        return STG_E_INVALID;
    }
    return download_fields(h, h->x64, p_out, vel_out);
}

// ---------------------------------------------------------------- energy
static int energy_input(stg_t* h, const double* p, const double* const* vel, const d4** x) {
    if (!p && !vel) {
        if (!h->have_solution) {
            set_error("no device-resident solution");
            return STG_E_INVALID;
        }
        *x = h->x64;
        return STG_OK;
    }
    const double* dc = nullptr;
    const double* df[3] = {nullptr, nullptr, nullptr};
    STG_TRY(upload_fields(h, p, vel, &dc, df));
    STG_TRY(fields_to_vec(h, dc, df, h->r64));
    *x = h->r64;
    return STG_OK;
}

int stg_energy(stg_t* h, const double* p, const double* const* vel, double* J) {
    STG_TRY(check_handle(h));
    const d4* x;
    STG_TRY(energy_input(h, p, vel, &x));
    int nb = 0;
    STG_TRY(energy_op(h, x, h->t64, h->d_parts, &nb));
    STG_TRY(reduce_parts(h->st, h->d_parts, nb, h->dnrm));
    double s = 0;
    STG_CK(cudaMemcpyAsync(&s, h->dnrm, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    if (J) *J = 0.5 * s;
    return STG_OK;
}

int stg_energy_grad_x(stg_t* h, const double* p, const double* const* vel, double* p_grad, double* const* vel_grad) {
    STG_TRY(check_handle(h));
    const d4* x;
    STG_TRY(energy_input(h, p, vel, &x));
    int nb = 0;
    STG_TRY(energy_op(h, x, h->t64, nullptr, &nb));
    return download_fields(h, h->t64, p_grad, vel_grad);
}

int stg_energy_grad_q(stg_t* h, const double* p, const double* const* vel, double* cell_q, double* const* face_q) {
    STG_TRY(check_handle(h));
    const d4* x;
    STG_TRY(energy_input(h, p, vel, &x));
    // 1/2 x^2 per unknown (fluid_topo/FluidEnergy3D.cpp:82-91)
    STG_TRY(half_square64(h->st, h->n4, x, h->t64));
    return download_fields(h, h->t64, cell_q, face_q);
}

// ---------------------------------------------------------------- design loop
int stg_set_density(stg_t* h, const double* rho, const stg_alpha* law) {
    STG_TRY(check_handle(h));
    if (!law || !h->have_boundary) {
        set_error(!law ? "null alpha law" : "stg_set_boundary must come first");
        return STG_E_INVALID;
    }
    if (rho) STG_CK(cudaMemcpyAsync(h->d_phys, rho, sizeof(double) * h->ncell, cudaMemcpyHostToDevice, h->st));
    if (h->dim == 2) {
        STG_TRY(set_density2d(h, h->d_phys, *law));
    } else {
        Level& F = fine(h);
        STG_TRY(face_penalty_from_density(h->st, F.g, h->d_phys, *law, F.m, F.P64, F.P32));
    }
    h->have_penalty = true;
    h->updated = false;
    h->phys_used = h->d_phys;
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_adjoint_sensitivity(stg_t* h, const stg_alpha* law, double* dJ, stg_stats* stats) {
    STG_TRY(check_handle(h));
    if (!law || !h->have_solution || !h->phys_used) {
        set_error("needs an alpha law, a prior stg_solve and a density set by stg_set_density");
        return STG_E_INVALID;
    }
    // adjoint right-hand side E x, then A lambda = E x (A is symmetric)
    int nb = 0;
    STG_TRY(energy_op(h, h->x64, h->t64, nullptr, &nb));
    int rc = solve_core(h, h->t64, h->lam64, stats);
    if (rc == STG_OK || rc == STG_E_NOT_CONVERGED) h->x0_valid[1] = true;
    if (rc != STG_OK && rc != STG_E_NOT_CONVERGED) return rc;
    if (h->dim == 2)
        STG_TRY(sensitivity2d(h, h->phys_used, *law, h->x64, h->lam64, h->d_sens));
    else
        STG_TRY(sensitivity(h->st, fine(h).g, h->phys_used, *law, h->x64, h->lam64, h->d_sens));
    if (dJ) STG_CK(cudaMemcpyAsync(dJ, h->d_sens, sizeof(double) * h->ncell, cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    return rc;
}

int stg_filter(stg_t* h, double rmin, const double* in, double* out, int transpose) {
    STG_TRY(check_handle(h));
    if (!(rmin > 0)) {
        set_error("rmin must be positive");
        return STG_E_INVALID;
    }
    double* src = transpose ? h->d_sens : h->d_design;
    double* dst = transpose ? h->d_sens_design : h->d_phys;
    if (in) {
        STG_CK(cudaMemcpyAsync(h->d_tmp, in, sizeof(double) * h->ncell, cudaMemcpyHostToDevice, h->st));
        src = h->d_tmp;
    }
    STG_TRY(density_filter(h->st, h->dim, h->n, rmin, src, dst, transpose, h->d_wsum));
    if (out) STG_CK(cudaMemcpyAsync(out, dst, sizeof(double) * h->ncell, cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_oc_update(stg_t* h, double rmin, const double* x, const double* dc, double frac, double move, double lo, double hi,
                  double* x_new, double* lambda_out) {
    STG_TRY(check_handle(h));
    const int nc = (int)h->ncell;
    if (h->vw_rmin != rmin) {
        // vw_j = sum_i w_ij / W_i: the filtered volume is sum_j vw_j x_j
        std::vector<double> ones(h->ncell, 1.0);
        STG_CK(cudaMemcpyAsync(h->d_tmp, ones.data(), sizeof(double) * h->ncell, cudaMemcpyHostToDevice, h->st));
        STG_TRY(density_filter(h->st, h->dim, h->n, rmin, h->d_tmp, h->d_vw, 1, h->d_wsum));
        STG_CK(cudaStreamSynchronize(h->st));
        h->vw_rmin = rmin;
    }
    if (x) STG_CK(cudaMemcpyAsync(h->d_design, x, sizeof(double) * h->ncell, cudaMemcpyHostToDevice, h->st));
    const double* ddc = h->d_sens_design;
    if (dc) {
        STG_CK(cudaMemcpyAsync(h->d_sens, dc, sizeof(double) * h->ncell, cudaMemcpyHostToDevice, h->st));
        ddc = h->d_sens;
    }
    // the multiplier grows with the sensitivities (with the objective, i.e. with the grid:
    // above 1e9 at 512^3): the bracket is widened by decades until its upper end
    // undershoots, then bisected - all of it in one cooperative launch, with no host
    // round trip per multiplier step
    STG_TRY(oc_update_device(h->st, nc, h->d_design, ddc, h->d_vw, frac, move, lo, hi, h->d_tmp, h->d_parts, h->dnrm));
    STG_CK(cudaMemcpyAsync(h->d_design, h->d_tmp, sizeof(double) * h->ncell, cudaMemcpyDeviceToDevice, h->st));
    if (x_new) STG_CK(cudaMemcpyAsync(x_new, h->d_design, sizeof(double) * h->ncell, cudaMemcpyDeviceToHost, h->st));
    double lmid = 0;
    STG_CK(cudaMemcpyAsync(&lmid, h->dnrm, sizeof(double), cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    if (lambda_out) *lambda_out = lmid;
    return STG_OK;
}

int stg_mma_update(stg_t* h, const double* x, const double* dfdx, double frac, double coef, double lo, double hi, double move,
                   double* x_new, double* change) {
    STG_TRY(check_handle(h));
    if (!(hi > lo) || !(move > 0)) {
        set_error("MMA bounds need hi > lo and move > 0");
        return STG_E_INVALID;
    }
    if (x) STG_CK(cudaMemcpyAsync(h->d_design, x, sizeof(double) * h->ncell, cudaMemcpyHostToDevice, h->st));
    const double* ddf = h->d_sens_design;
    if (dfdx) {
        STG_CK(cudaMemcpyAsync(h->d_sens, dfdx, sizeof(double) * h->ncell, cudaMemcpyHostToDevice, h->st));
        ddf = h->d_sens;
    }
    double ch = 0;
    STG_TRY(mma_update(h, h->d_design, ddf, frac, coef, lo, hi, move, h->d_tmp, &ch));
    STG_CK(cudaMemcpyAsync(h->d_design, h->d_tmp, sizeof(double) * h->ncell, cudaMemcpyDeviceToDevice, h->st));
    if (x_new) STG_CK(cudaMemcpyAsync(x_new, h->d_design, sizeof(double) * h->ncell, cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    if (change) *change = ch;
    return STG_OK;
}

int stg_mma_reset(stg_t* h) {
    STG_TRY(check_handle(h));
    return mma_reset(h);
}

int stg_density_noise(stg_t* h, uint64_t seed, double sigma, double* out) {
    STG_TRY(check_handle(h));
    int R = -1;
    if (sigma > 0) {
        R = (int)std::ceil(3.0 * sigma);
        if (2 * R + 1 > 512) {
            set_error("sigma too large");
            return STG_E_INVALID;
        }
        std::vector<double> w(2 * R + 1);
        double s = 0;
        for (int t = -R; t <= R; t++) s += (w[t + R] = std::exp(-(double)(t * t) / (2.0 * sigma * sigma)));
        for (auto& v : w) v /= s;
        STG_CK(cudaMemcpyAsync(h->d_gauss, w.data(), sizeof(double) * w.size(), cudaMemcpyHostToDevice, h->st));
    }
    STG_TRY(density_noise(h->st, h->dim, h->n, seed, h->d_gauss, R, h->d_design, h->d_tmp));
    if (out) STG_CK(cudaMemcpyAsync(out, h->d_design, sizeof(double) * h->ncell, cudaMemcpyDeviceToHost, h->st));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

// ---------------------------------------------------------------- LinearMapping adapters
int stg_apply_A_device(stg_t* h, int level, double* d_Ap, const double* d_p) {
    STG_TRY(check_handle(h));
    if (level < 0 || level >= h->L || !d_Ap || !d_p) {
        set_error("bad level or pointer");
        return STG_E_INVALID;
    }
    if (level < h->L - 1) STG_TRY(ensure_setup(h, true));
    if (h->dim == 2) {
        STG_TRY(apply_A2d(h, level, d_Ap, d_p));
        STG_CK(cudaStreamSynchronize(h->st));
        return STG_OK;
    }
    Level& L = h->lv[level];
    STG_TRY(ensure_adapter(L));
    STG_TRY(blocked_to_slots64(h->st, L.g, d_p, L.t0));
    if (h->gen)
        STG_TRY(op64v(h->st, L.g, L.t0, L.m, L.P64, L.V64, nullptr, L.t1, 0, nullptr, nullptr));
    else
        STG_TRY(op64(h->st, L.g, L.vol, L.t0, L.m, L.P64, nullptr, L.t1, 0, nullptr, nullptr));
    // padding entries of the reference layout are fixed identity rows
    STG_TRY(slots_to_blocked64(h->st, L.g, L.t1, d_Ap, d_p));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_apply_E_device(stg_t* h, double* d_Ap, const double* d_p) {
    STG_TRY(check_handle(h));
    if (h->dim == 2) {
        STG_TRY(apply_E2d(h, d_Ap, d_p));
        STG_CK(cudaStreamSynchronize(h->st));
        return STG_OK;
    }
    Level& L = fine(h);
    STG_TRY(ensure_adapter(L));
    STG_TRY(blocked_to_slots64(h->st, L.g, d_p, L.t0));
    if (h->gen)
        STG_TRY(op64v(h->st, L.g, L.t0, L.m, L.P64, L.V64, nullptr, L.t1, 2, nullptr, nullptr));
    else
        STG_TRY(op64(h->st, L.g, L.vol, L.t0, L.m, L.P64, nullptr, L.t1, 2, nullptr, nullptr));
    STG_TRY(slots_to_blocked64(h->st, L.g, L.t1, d_Ap, nullptr));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_update(stg_t* h) {
    STG_TRY(check_handle(h));
    h->hier_flow = false;  // FluidSteadyState3D::update: the reference's hierarchy
    STG_TRY(h->setup(h));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_vcycle_device(stg_t* h, double* d_out, const double* d_in) {
    STG_TRY(check_handle(h));
    STG_TRY(ensure_setup(h, true));
    if (h->dim == 2) {
        STG_TRY(vcycle2d(h, d_out, d_in));
        STG_CK(cudaStreamSynchronize(h->st));
        return STG_OK;
    }
    Level& F = fine(h);
    STG_TRY(ensure_adapter(F));
    STG_TRY(blocked_to_slots64(h->st, F.g, d_in, F.t0));
    if (h->gen) {
        STG_CK(cudaMemcpyAsync(F.gr, F.t0, sizeof(d4) * F.g.nslot, cudaMemcpyDeviceToDevice, h->st));
        STG_TRY(gen_vcycle(h));
        STG_TRY(slots_to_blocked64(h->st, F.g, F.gx, d_out, nullptr));
        STG_CK(cudaStreamSynchronize(h->st));
        return STG_OK;
    }
    PathGuard guard{h};
    STG_TRY(choose_path(h, F, F.t0));
    STG_TRY(f64_to_f32(h->st, F.g.nslot, F.t0, 1.0, h->w));
    STG_TRY(vcycle(h, h->w));
    STG_TRY(f32_to_f64(h->st, F.g.nslot, F.x(), F.t1));
    STG_TRY(slots_to_blocked64(h->st, F.g, F.t1, d_out, nullptr));
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

int stg_apply_op_device(stg_t* h, int op, int level, double* d_out, const double* d_in) {
    STG_TRY(check_handle(h));
    if (level < 0 || level >= h->L || !d_out || !d_in) {
        set_error("bad level or pointer");
        return STG_E_INVALID;
    }
    STG_TRY(ensure_setup(h, true));
    if (h->dim == 2) {
        STG_TRY(apply_op2d(h, op, level, d_out, d_in));
        STG_CK(cudaStreamSynchronize(h->st));
        return STG_OK;
    }
    Level& L = h->lv[level];
    STG_TRY(ensure_adapter(L));
    switch (op) {
        case STG_OP_RESTRICT: {
            if (level >= h->L - 1) break;
            Level& F = h->lv[level + 1];
            STG_TRY(ensure_adapter(F));
            STG_TRY(blocked_to_slots64(h->st, F.g, d_in, F.t0));
            STG_TRY(restrict64(h->st, L.g, F.g, F.t0, L.m, L.t1));
            STG_TRY(slots_to_blocked64(h->st, L.g, L.t1, d_out, nullptr));
            STG_CK(cudaStreamSynchronize(h->st));
            return STG_OK;
        }
        case STG_OP_PROLONG: {
            if (level >= h->L - 1) break;
            Level& F = h->lv[level + 1];
            STG_TRY(ensure_adapter(F));
            STG_TRY(blocked_to_slots64(h->st, L.g, d_in, L.t0));
            STG_TRY(prolong64(h->st, F.g, L.g, L.t0, F.m, F.t1));
            STG_TRY(slots_to_blocked64(h->st, F.g, F.t1, d_out, nullptr));
            STG_CK(cudaStreamSynchronize(h->st));
            return STG_OK;
        }
        case STG_OP_SMOOTH_PRE:
        case STG_OP_SMOOTH_POST:
        case STG_OP_VANKA_RED:
        case STG_OP_VANKA_BLACK: {
            if (level == 0) break;
            STG_TRY(blocked_to_slots64(h->st, L.g, d_in, L.t0));
            if (h->gen) {
                if (op == STG_OP_SMOOTH_PRE || op == STG_OP_SMOOTH_POST)
                    STG_TRY(gen_smooth(h, L, op == STG_OP_SMOOTH_POST, L.t0, L.t1));
                else
                    STG_TRY(gen_vanka(h, L, op == STG_OP_VANKA_BLACK ? 1 : 0, L.t0, L.t1));
                STG_TRY(slots_to_blocked64(h->st, L.g, L.t1, d_out, nullptr));
                STG_CK(cudaStreamSynchronize(h->st));
                return STG_OK;
            }
            PathGuard guard{h};
            STG_TRY(choose_path(h, L, L.t0));
            STG_TRY(f64_to_f32(h->st, L.g.nslot, L.t0, 1.0, L.r));
            L.cur = 0;
            if (op == STG_OP_SMOOTH_PRE || op == STG_OP_SMOOTH_POST) {
                STG_CK(cudaMemsetAsync(L.x(), 0, sizeof(float4) * L.g.nslot, h->st));
                STG_TRY(smooth(h, L, L.r, op == STG_OP_SMOOTH_POST, true));
            } else {
                STG_TRY(sweep32(h->st, L.g, (float)L.vol, L.r, nullptr, L.x(), L.m, L.P32, op == STG_OP_VANKA_BLACK ? 1 : 0,
                                fast(h, L)));
            }
            STG_TRY(f32_to_f64(h->st, L.g.nslot, L.x(), L.t1));
            STG_TRY(slots_to_blocked64(h->st, L.g, L.t1, d_out, nullptr));
            STG_CK(cudaStreamSynchronize(h->st));
            return STG_OK;
        }
        case STG_OP_COARSE: {
            if (level != 0) break;
            STG_TRY(blocked_to_slots64(h->st, L.g, d_in, L.t0));
            STG_TRY(dense_apply64(h->st, h->dense, L.g, L.t0, L.t1));
            // padding entries of the reference layout are fixed identity rows of its matrix
            STG_TRY(slots_to_blocked64(h->st, L.g, L.t1, d_out, d_in));
            STG_CK(cudaStreamSynchronize(h->st));
            return STG_OK;
        }
        default: break;
    }
    set_error("operator %d not defined at level %d", op, level);
    return STG_E_INVALID;
}

int stg_level_descr_device(stg_t* h, int level, double* d_vol, double* d_penalty, uint8_t* d_fixed) {
    STG_TRY(check_handle(h));
    if (level < 0 || level >= h->L) {
        set_error("bad level");
        return STG_E_INVALID;
    }
    STG_TRY(ensure_setup(h, true));
    if (h->dim == 2) {
        STG_TRY(level_descr2d(h, level, d_vol, d_penalty, d_fixed));
        STG_CK(cudaStreamSynchronize(h->st));
        return STG_OK;
    }
    Level& L = h->lv[level];
    STG_TRY(ensure_adapter(L));
    if (d_penalty) STG_TRY(slots_to_blocked64(h->st, L.g, L.P64, d_penalty, nullptr));
    if (d_fixed) STG_TRY(mask_to_blocked(h->st, L.g, L.m, d_fixed));
    if (d_vol) {
        if (h->gen) {
            STG_TRY(slots_to_blocked64(h->st, L.g, L.V64, d_vol, nullptr));
        } else {
            STG_TRY(vol_slots(h->st, L.g, L.m, L.cell_vol, L.vol, L.t0));
            STG_TRY(slots_to_blocked64(h->st, L.g, L.t0, d_vol, nullptr));
        }
    }
    STG_CK(cudaStreamSynchronize(h->st));
    return STG_OK;
}

}  // extern "C"
