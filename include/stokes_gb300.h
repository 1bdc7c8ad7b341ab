/*
 * stokes_gb300.h - C ABI of the GB300 Brinkman-Stokes topology-optimization hot path.
 *
 * One handle owns one problem on one GPU: the multigrid hierarchy, the Krylov
 * workspace and the design-loop buffers, all resident in device memory. Every call
 * returns 0 on success and a negative STG_E_* code on failure; stg_last_error()
 * gives the message of the last failure on the calling thread. A handle is used by
 * one host thread at a time and issues its work on its own CUDA stream.
 *
 * Host arrays use the simplex Field order of the reference
 * (simplex/src/reservoir/Field.h:67-72): a 3D cell array has N^3 entries with cell
 * (i,j,k) at (i*N + j)*N + k; face axis d is a separate array with N+1 entries along
 * d (simplex/src/reservoir/FaceField.h:16), so Field::array.data() plugs in directly.
 * 2D arrays follow the same rule with (i*N + j).
 *
 * "Blocked" device vectors use the reference solver layout
 * [cells | x-faces | y-faces | z-faces] of common_cpx/grid3D.cu:24-146 (3D) and
 * [cells | x-faces | y-faces] of common_cpx/form01mapping.cu:10-57 (2D), so the
 * device-pointer entry points can sit behind the reference LinearMapping interface
 * (common_cpx/LinearMapping.h:4-14) unchanged.
 */
#ifndef STOKES_GB300_H
#define STOKES_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define STG_OK 0
#define STG_E_INVALID (-1)     /* bad argument, size or state */
#define STG_E_CUDA (-2)        /* a CUDA call failed */
#define STG_E_NOMEM (-3)       /* device allocation failed */
#define STG_E_UNSUPPORTED (-4) /* input outside what this build implements */
#define STG_E_NOT_CONVERGED (-5)
#define STG_E_NONFINITE (-6) /* NaN/Inf met in a residual */

typedef struct stg_ctx stg_t;

/* Solver method of stg_solve. */
#define STG_METHOD_PLAIN 0 /* FP32 V-cycle preconditioned FGMRES inside FP64 refinement */
#define STG_METHOD_MIXED 1 /* as PLAIN with BF16-stored coarse-level corrections */
#define STG_METHOD_LEARNED 2 /* as PLAIN with the learned correction of stg_net_* added to every
                                V-cycle; falls back to PLAIN for the rest of a solve when a
                                Krylov step other than the first of a refinement step reduces
                                the residual estimate by less than 20% */

typedef struct stg_opts {
    int method;          /* STG_METHOD_* */
    double tol;          /* FP64 true relative residual ||b-Ax||/||b|| to reach */
    int max_outer;       /* FP64 refinement steps */
    int inner_max;       /* FGMRES basis size of one refinement step (2D: at least 60) */
    double inner_tol;    /* relative reduction asked of one refinement step */
    int verbose;         /* print per-iteration residuals to stderr */
    int smooth_sweeps;   /* sweeps per colour in the solver's smoother: 1 (default; 0 means
                            1) or 2, the reference's DescentSmoother. At 256^3 one sweep per
                            colour reaches the same FP64 tolerance in as many V-cycles at
                            2/3 of the time. A refinement step that uses the whole basis
                            without reaching its target raises it to 2 for the rest of
                            the solve and for the handle's next solve (3D). The
                            LinearMapping adapters always run the reference smoother. */
    int warm_start;      /* 1: start each solve from the previous solution of the same
                            equation (the forward one for stg_solve, the adjoint one for
                            stg_adjoint_sensitivity) instead of zero, unless its residual
                            exceeds ||b|| (then zero); 2: the same, then a learned
                            correction of that start (3D, needs a network: one FGMRES step
                            whose preconditioner is the network-corrected V-cycle, its
                            length minimising the residual); 0 (default): zero, as the
                            reference */
    int prolong;         /* coarse-correction transfer of the 3D solver's uniform-form V-cycle:
                            0 the reference's piecewise-constant injection
                            (StokeFlowUpSample3D); 1 face velocities interpolated - linearly
                            along the face normal, 3/4 : 1/4 between the two nearest coarse
                            faces along each tangent - and pressures injected. The
                            LinearMapping adapters always inject. */
    int basis16;         /* 1 (default): the 3D uniform-form FGMRES also keeps an FP16 copy
                            of each basis vector (8 more bytes per slot and vector), from
                            which its multi-dot pass reads; the projections and the
                            solution update keep the FP32 basis. Where the copies do not
                            fit in device memory the handle runs without them. 0: FP32
                            only (e.g. to fit a 512^3 solve with a long basis in a memory
                            budget). */
} stg_opts;

typedef struct stg_stats {
    int outer_iters;     /* FP64 refinement steps taken */
    int inner_iters;     /* total FGMRES iterations (= V-cycles) */
    double rel_residual; /* final FP64 true relative residual */
    double abs_residual;
    double setup_ms;     /* hierarchy + coarsest-inverse set-up time */
    double solve_ms;     /* device time of the Krylov solve */
    int status;          /* 0 converged, STG_E_* otherwise */
    int learned_iters;   /* FGMRES iterations whose preconditioner added the learned correction */
    int fallbacks;       /* refinement steps that fell back from LEARNED to PLAIN after a stall */
} stg_stats;

/* Runs the handle's work on a caller-owned CUDA stream (a cudaStream_t passed as void*);
 * NULL returns to the handle's own stream. Not part of the reference, which uses the
 * default stream. */
int stg_set_stream(stg_t* h, void* cuda_stream);

/* Kernel accounting: total kernels this library has launched in the process, and
 * per-kernel-class CUDA-event timing on the handle's stream (off by default). Classes:
 * 0 resid32, 1 sweep32 (finest level), 2 restrict32, 3 prolong32, 4 apply32, 5 resid64,
 * 6 krylov, 7 coarse, 8 setup, 9 other, 10 sweep32_coarse (coarser levels), 11 net
 * (the learned correction's network). */
#define STG_PROF_NCLASS 12
int64_t stg_kernel_launches(void);
int stg_profile(stg_t* h, int enable); /* enabling also clears the counters */
int stg_profile_read(stg_t* h, int cls, int64_t* launches, double* ms, double* bytes);
const char* stg_profile_name(int cls);

/* Fills *o with the defaults (PLAIN, tol 1e-8, 20 outer, 30 inner, 1e-4, 1 sweep per colour,
   no warm start, injection, FP16 basis copies). */
void stg_default_opts(stg_opts* o);

/* Message of the last failure on this thread ("" if none). */
const char* stg_last_error(void);

/* Library build string (arch, version). */
const char* stg_version(void);

/* ----------------------------------------------------------------------------
 * Solver-class API: FluidSteadyState3D / FluidSteadyState
 * (stoke/FluidSteadyState3D.h:11-38, stoke/FluidSteadyState.h).
 * -------------------------------------------------------------------------- */

/* FluidSteadyState3D::init(N) (stoke/FluidSteadyState3D.cpp:12-90), dim 3: levels =
 * log2(lowbit N) - 1, N a multiple of 4 in [4, 1024]. FluidSteadyState::init(N)
 * (stoke/FluidSteadyState.cpp:9-85), dim 2: levels = log2(lowbit N) - 2, N a multiple of
 * 8 up to 16384 whose coarsest level has at most 8192 unknowns. */
int stg_create(int dim, int n, const stg_opts* opts, stg_t** out);
int stg_destroy(stg_t* h);

/* Number of levels and cells per axis of a level (level 0 = coarsest, as the reference). */
/* Switches the solver method of a handle (STG_METHOD_*; LEARNED needs dim 3). */
int stg_set_method(stg_t* h, int method);
int stg_levels(const stg_t* h);
int stg_level_n(const stg_t* h, int level);
/* LinearMapping::xDoF()/yDoF() of the reference operator at a level (blocked layout size). */
int64_t stg_level_dof(const stg_t* h, int level);

/* FluidSteadyState3D::init_boundary(cell_vol, cell_fixed, face_vol, face_fixed, closed)
 * (stoke/FluidSteadyState3D.cpp:92-114) together with FluidEnergy3D::init_boundary
 * (fluid_topo/FluidEnergy3D.cpp:33-54); 2D: FluidSteadyState::init_boundary
 * (stoke/FluidSteadyState.cpp:87-108). face_* point to dim arrays. Any vol and fixed
 * flags are accepted. In 3D, when the free faces share one vol value and no cell is
 * fixed, the solver uses its uniform-coefficient form (closed-form Vanka blocks, FP32
 * V-cycle; with every face on the domain boundary fixed, as in every reference test, the
 * 7-point Laplacian form of the same matrix); otherwise the general-coefficient form
 * (per-face vols, Vanka blocks probed and LU-factored like the reference's, FP64
 * V-cycle), which STG_METHOD_LEARNED does not support. With fixed cells the reference's
 * own coarsest matrix is singular; this library adds the fixed cells' identity rows. */
int stg_set_boundary(stg_t* h, const double* cell_vol, const int32_t* cell_fixed, const double* const* face_vol,
                     const int32_t* const* face_fixed, int closed);

/* FluidSteadyState3D::update_penalty(cell_penalty, face_penalty) (:130-150) and
 * FluidEnergy3D::update_penalty. cell_penalty may be NULL (zero). */
int stg_set_penalty(stg_t* h, const double* cell_penalty, const double* const* face_penalty);

/* FluidSteadyState3D::update_b(cell_b, face_b) (:116-127). Returns once the host arrays
 * have been read. In 3D, a set-up pending since the last penalty change runs while b is
 * copied, and the next stg_solve uses it instead of repeating it. */
int stg_set_rhs(stg_t* h, const double* cell_b, const double* const* face_b);

/* FluidSteadyState3D::solve() (:152-170): coarse re-discretisation, smoother and
 * coarsest set-up (unless stg_set_rhs ran it after the last penalty change), then the
 * Krylov solve from a zero initial guess (or the previous solution, stg_opts.warm_start). The results go to
 * p_out (cells) and vel_out[dim] (faces), the public members p and vel of the
 * reference; either may be NULL to keep the solution on the device only.
 * The solver's own coarse levels differ from the reference's in one rule: a coarse
 * velocity unknown carries 2^dim x the smallest penalty of its free children, not their
 * sum, so that channels narrower than a coarse cell stay open on the coarse levels (with
 * the sum, solves on optimised high-contrast designs stagnate). The adapters below
 * (stg_update, stg_vcycle_device, stg_apply_op_device, stg_level_descr_device) keep the
 * reference's sums; the two set-ups replace each other as the calls alternate. */
int stg_solve(stg_t* h, double* p_out, double* const* vel_out, stg_stats* stats);

/* Copies the last solution to host Field arrays. */
int stg_get_solution(stg_t* h, double* p_out, double* const* vel_out);

/* ----------------------------------------------------------------------------
 * Energy API: FluidEnergy3D (fluid_topo/FluidEnergy3D.h:10-44).
 * The velocity/pressure arguments are host Field arrays; NULL means "use the last
 * solution held on the device".
 * -------------------------------------------------------------------------- */

/* compute_energy(vel, p): J = 1/2 x^T E x (fluid_topo/FluidEnergy3D.cpp:94-109). */
int stg_energy(stg_t* h, const double* p, const double* const* vel, double* J);
/* compute_gradient_x(vel, p): p_grad, vel_grad = E x (:71-80). */
int stg_energy_grad_x(stg_t* h, const double* p, const double* const* vel, double* p_grad, double* const* vel_grad);
/* compute_gradient_q(vel, p): 1/2 x^2 per DOF (:82-91). */
int stg_energy_grad_q(stg_t* h, const double* p, const double* const* vel, double* cell_q, double* const* face_q);

/* ----------------------------------------------------------------------------
 * Design-loop API (FluidTopoOpt3D, fluid_topo/FluidTopoOpt3D.cpp:4-223, plus the
 * density filter and optimality-criteria update of the target problem).
 * -------------------------------------------------------------------------- */

#define STG_ALPHA_REF 0 /* alpha_os + (alpha_us - alpha_os) s (1+q)/(s+q), s = rho^3 (FluidTopoOpt3D.cpp:110-123) */
#define STG_ALPHA_BP 1  /* amax * 0.1 (1 - rho)/(0.1 + rho) on the filtered density */

typedef struct stg_alpha {
    int law;         /* STG_ALPHA_* */
    double alpha_os; /* REF: solid value (the reference scales 5e2 by 32/N) */
    double alpha_us; /* REF: fluid value (1e-3) */
    double q;        /* REF: 0.01 in 3D, 0.014 in 2D */
    double amax;     /* BP: 1e4 */
} stg_alpha;

/* Update_Fluid's penalty assembly (FluidTopoOpt3D.cpp:145-159) on the GPU: face
 * penalty = sum over the adjacent cells of 1/2 alpha(rho_c); installs it as with
 * stg_set_penalty (cell penalty zero). rho: host cell array, or NULL to use the
 * device-resident design of stg_filter. */
int stg_set_density(stg_t* h, const double* rho, const stg_alpha* law);

/* Adjoint sensitivity (FluidTopoOpt3D::Update_Grad, :170-198): solves A lambda = E x
 * with the same solver, then dJ/drho_c = 1/2 alpha'(.) (ds/drho) sum_{faces of c}
 * (-u_f lambda_f + 1/2 u_f^2). Needs a prior stg_solve. dJ (host, N^dim) may be NULL
 * to keep the result on the device. */
int stg_adjoint_sensitivity(stg_t* h, const stg_alpha* law, double* dJ, stg_stats* stats);

/* Linear hat density filter of radius rmin cells: rho~ = H rho, weights
 * max(0, rmin - |c_i - c_j|) normalised per row. in/out are host cell arrays; out NULL
 * keeps the filtered design on the device for stg_set_density. transpose != 0 applies
 * H^T (sensitivity chain rule). */
int stg_filter(stg_t* h, double rmin, const double* in, double* out, int transpose);

/* Optimality-criteria update with a bisection on the volume multiplier:
 * x_new = clamp(x sqrt(max(0,-dc)/(lambda dv)), max(lo, x - move), min(hi, x + move)),
 * with the volume of the filtered design equal to frac. x, dc host arrays (NULL:
 * device-resident design / sensitivity); x_new may alias x. */
int stg_oc_update(stg_t* h, double rmin, const double* x, const double* dc, double frac, double move, double lo, double hi,
                  double* x_new, double* lambda_out);

/* One design update of the reference optimizer: the loop body of
 * OptimizerMMA::Optimize_MMA (simplex/src/optimization/OptimizerMma.h:96-128), i.e. the
 * Method of Moving Asymptotes of simplex/ext/mma/MMASolver.cpp (dual interior point), with
 * the volume constraint of FluidTopoOpt3D::Compute_Constraint(_Grad)
 * (fluid_topo/FluidTopoOpt3D.cpp:19-39): g = coef (mean x - frac), dg/dx = coef / ncell,
 * and per-cell bounds [max(lo, x - move), min(hi, x + move)] (the reference: coef 1e4,
 * lo 0.01, hi 1, move 0.2). The asymptotes carry over between calls (stg_mma_reset starts
 * a new run, as a new MMASolver does). x: host design, or NULL for the device-resident
 * design; dfdx: host gradient, or NULL for the device sensitivity left by
 * stg_filter(..., transpose = 1). x_new (host, may alias x, or NULL) receives the new
 * design, which also stays on the device; change: max |x_new - x|, the reference's
 * stopping quantity. */
int stg_mma_update(stg_t* h, const double* x, const double* dfdx, double frac, double coef, double lo, double hi, double move,
                   double* x_new, double* change);
int stg_mma_reset(stg_t* h);

/* The optimality-criteria update of stg_oc_update for callers that cannot allocate
 * device memory: applications that reserve the whole GPU for their own pool, plugins
 * running under another framework's allocator budget, and latency-sensitive loops that
 * cannot afford the device-wide synchronisation of cudaMalloc/cudaFree. No counterpart
 * in the reference. The caller passes device arrays of N^3 cells (Field order): the
 * design d_x, the sensitivity d_dc and the result d_xnew (which may alias d_x); no
 * handle is needed and nothing is allocated.
 * The only scratch is a fixed 42 KB array inside this library's device image (every GPU
 * that loads the library holds it until exit). All calls share the array, so calls that overlap on the GPU (other streams, other host
 * threads on the same device) race; serialise them. N above 1024 and filter radii rmin
 * above 4 are rejected with STG_E_INVALID. Work is issued on cuda_stream (a cudaStream_t,
 * NULL = legacy default stream) and synchronised before return. Results equal
 * stg_oc_update's. */
int stg_oc_update_noalloc(int n, double rmin, const double* d_x, const double* d_dc, double frac, double move, double lo,
                          double hi, double* d_xnew, double* lambda_out, void* cuda_stream);

/* ----------------------------------------------------------------------------
 * LinearMapping plugin API (common_cpx/LinearMapping.h:4-14) on raw device pointers in
 * the reference blocked layout; issued on the handle's stream and synchronised
 * before return.
 * -------------------------------------------------------------------------- */

/* StokeFlowMapping3DFixed::applyMapping(Ap, p) at a level (stoke/StokeFlowMapping3D.cu:218-348), FP64. */
int stg_apply_A_device(stg_t* h, int level, double* d_Ap, const double* d_p);
/* FluidEnergyGrad3D::applyMapping(Ap, p) (fluid_topo/FluidEnergyGrad3D.cu:201-308), FP64. */
int stg_apply_E_device(stg_t* h, double* d_Ap, const double* d_p);
/* MultigridSolve::update() (common_cpx/MultigridSolve.cpp:116-124) together with the coarse
 * re-discretisation of FluidSteadyState3D::solve (:155). */
int stg_update(stg_t* h);
/* MultigridSolve::applyMapping(Ap, p) (common_cpx/MultigridSolve.cpp:108-114): one V-cycle
 * from a zero guess, FP32 arithmetic inside, FP64 in and out. */
int stg_vcycle_device(stg_t* h, double* d_out, const double* d_in);

/* Component entry points behind the same interface (one LinearMapping each):
 *  STG_OP_RESTRICT   StokeFlowDownSample3D (stoke/StokeFlowSubSystem3D.cu:32-52), level = coarse level
 *  STG_OP_PROLONG    StokeFlowUpSample3D   (:81-101), level = coarse level
 *  STG_OP_SMOOTH_PRE / STG_OP_SMOOTH_POST  DescentSmoother of StokeLike::GenerateJacobiPreconditioner
 *                    (stoke/StokeLike.cu:345-372, common_cpx/DescentSmoother.cu:31-47)
 *  STG_OP_VANKA_RED / STG_OP_VANKA_BLACK   VelDiagPressureFullSmoothing (stoke/StokeLike.cu:220-278)
 *  STG_OP_COARSE     DirectSolve3D::applyMapping (stoke/StokeLike.cu:421-425), level 0
 * The smoothing and coarse operators compute in FP32 (coarse: FP64) with FP64 in/out. */
#define STG_OP_RESTRICT 1
#define STG_OP_PROLONG 2
#define STG_OP_SMOOTH_PRE 3
#define STG_OP_SMOOTH_POST 4
#define STG_OP_VANKA_RED 5
#define STG_OP_VANKA_BLACK 6
#define STG_OP_COARSE 7
int stg_apply_op_device(stg_t* h, int op, int level, double* d_out, const double* d_in);

/* Coarse descriptor of a level after stg_update (StokeFlowDescriptor3D d_vol,
 * d_penalty, d_fixed; stoke/StokeFlowDescriptor3D.h:5-30), blocked layout, device pointers. */
int stg_level_descr_device(stg_t* h, int level, double* d_vol, double* d_penalty, uint8_t* d_fixed);

/* ----------------------------------------------------------------------------
 * Learned preconditioner (not part of the reference): a 3-level 3D U-Net (16/32/64
 * channels, 3x3x3 convolutions, BF16 weights and activations, FP32 accumulation on the
 * tensor cores) that maps (density, face penalties, residual after a V-cycle) to a
 * correction. STG_METHOD_LEARNED uses it inside FGMRES as z = M(v) + NN(v - A M(v)).
 * Parameters are one FP32 vector: per convolution l = 0..9 the weights [27][C_out][C_in]
 * (tap 9 (di+1) + 3 (dj+1) + (dk+1)) then the biases [C_out]; the 1x1 head [4][16] and its
 * biases [4]; last, the output scale kappa (set by the first training pair, not trained).
 * -------------------------------------------------------------------------- */

/* Creates the handle's network (or re-initialises it) with seeded He-uniform weights. */
int stg_net_init(stg_t* h, uint64_t seed);
int stg_net_num_params(const stg_t* h, int64_t* count);
int stg_net_get_params(stg_t* h, float* out, int64_t count);
/* Loads parameters and resets the Adam state. */
int stg_net_set_params(stg_t* h, const float* in, int64_t count);
/* One forward pass on host data of an n^3 grid (n >= 8, n % 4 == 0), independent of the
 * handle's grid: in [n^3][8] channels (density, p, u, v, w, three penalty shares), cell
 * v = (i n + j) n + k. out [n^3][4] (may be NULL). With target [n^3][4] non-NULL, also the
 * loss sum (out - target)^2 / sum target^2 and its gradient with respect to every
 * parameter (grad may be NULL), kept for stg_net_adam_step. */
int stg_net_forward_backward(stg_t* h, int n, const float* in, const float* target, float* out, float* grad, double* loss);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) with the last computed gradient. */
int stg_net_adam_step(stg_t* h, double lr);
/* Trains on the handle's current operator (3D; boundary and penalty or density set):
 * each step draws a pair from seeded noise (e = M(noise), r = A e, z = M(r); input
 * r1 = r - A z, target e - z), runs forward, backward and Adam. losses: steps entries or NULL. */
int stg_net_train(stg_t* h, int steps, double lr, uint64_t seed, float* losses);

/* ----------------------------------------------------------------------------
 * Input generators used by the benchmarks (not part of the reference).
 * -------------------------------------------------------------------------- */

/* Seeded density: U[0,1) per cell keyed by (seed, Field index) through a SplitMix64
 * hash, separable Gaussian blur (sigma cells, truncated at ceil(3 sigma), clamp-to-edge)
 * along axes 0,1,2, clipped to [0,1]. Computed on the GPU; out is a host cell array,
 * or NULL to keep it as the handle's device-resident design. */
int stg_density_noise(stg_t* h, uint64_t seed, double sigma, double* out);

#ifdef __cplusplus
}
#endif
#endif /* STOKES_GB300_H */
