/*
 * sem_gb300.h -- C ABI of the GB300 (sm_103a) spectral-element library.
 *
 * This is the drop-in boundary for arotem3/SchrodingerSEM's hot path: the
 * matrix-free SEM operator apply, the element-interface gather-scatter and
 * Dirichlet masking, and the MINRES / PCG iterations behind the Poisson,
 * Helmholtz and Schroedinger (BDF2, SDIRK4 3-stage, SDIRK4 5-stage) solvers.
 * Each entry point names the reference interface it replaces (file:line in
 * the reference project).  The C++ layer in include/schro_gpu/ rebuilds the
 * reference's template API (minres, pcg, solver_results, solver_opts, ...)
 * on top of these calls.
 *
 * Conventions
 *  - A "field" is E*N*N doubles (N = p+1), element-contiguous, each element a
 *    column-major N x N block: value (i,j) of element e at e*N*N + j*N + i,
 *    i the xi index, j the eta index.  This is the memory of the reference's
 *    std::vector<arma::Mat<double>> laid end to end.
 *  - Field pointers of the operator-level calls (sem_unmask ... sem_pcg_*)
 *    are DEVICE pointers.  The driver-level calls (sem_poisson,
 *    sem_helmholtz, sem_schrodinger_*) accept host or device pointers and
 *    copy host data in and out themselves.
 *  - Every call returns an int status (SEM_OK = 0).  Solver non-convergence
 *    is not an error: it is reported in sem_solver_results.success or the
 *    driver's *success flag, as the reference does.
 *  - One context = one mesh + its device buffers, bound to one CUDA stream.
 *    Calls on one context are not reentrant.  Operator-level calls are
 *    asynchronous on that stream, except those that return a host scalar.
 */
#ifndef SEM_GB300_H
#define SEM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SEM_GB300_VERSION 1

/* status codes */
enum sem_status {
    SEM_OK = 0,
    SEM_ERR_ARG = 1,          /* bad argument (null pointer, size, degree out of range) */
    SEM_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    SEM_ERR_MESH = 3,         /* mesh topology invalid (bad corner id, not a quad mesh) */
    SEM_ERR_IO = 4,           /* mesh folder could not be read */
    SEM_ERR_DEVICE_WAIT = 5,  /* a device-side wait hit its time limit; results invalid */
    SEM_ERR_UNSUPPORTED = 6,  /* request outside what this build supports */
    SEM_ERR_NO_DEVICE = 7     /* no CUDA device visible */
};

/* context creation flags */
#define SEM_FLAG_METRIC_CORRECTED 0x1u /* C(i,j) = (Y_xi[j]^2 + X_xi[j]^2)/J.  Without this
                                          flag the reference's formula include/Quad.hpp:53
                                          (Y_xi[i]^2) is reproduced, for parity. */
#define SEM_FLAG_NEUMANN 0x2u /* natural (Neumann) boundary: boundary edges and corners
                                 stay degrees of freedom, owned by their first element and
                                 never masked (the reference zeroes them for Dirichlet data,
                                 include/mask_side.hpp:28-30, mask_node.hpp:13-21).  Every
                                 operator, solver and driver of the context follows it. */

/* options for sem_ctx_set_option */
enum sem_option {
    SEM_OPT_SOLVE_PRECISION = 1, /* SEM_PREC_FP64 (default) or SEM_PREC_MIXED */
    SEM_OPT_INNER_TOL = 2,       /* relative tolerance of the FP32 inner solve (default 1e-4) */
    SEM_OPT_STAGE_GUESS = 3,     /* SEM_GUESS_ZERO (reference), _EXTRAPOLATE, _LEARNED */
    SEM_OPT_WAIT_TIMEOUT_MS = 4, /* limit of every device-side wait (default 2000 ms) */
    SEM_OPT_MAX_REFINE = 5,      /* cap on FP64 refinement sweeps in mixed mode (default 50) */
    SEM_OPT_PROFILE = 6,         /* 1: time every persistent solver launch with CUDA events */
    SEM_OPT_PRECOND = 7,         /* preconditioner of the FP32 inner solve in mixed mode:
                                    SEM_PRECOND_NONE (default, as the reference),
                                    SEM_PRECOND_DIAG (diagonal of |A|) or SEM_PRECOND_FDM
                                    (Schroedinger Res only: per-element |A_e|^-1 by fast
                                    diagonalisation of the element's rectangle approximation,
                                    summed over elements with 1/multiplicity weights); the
                                    FP64 outer test on the true residual is unchanged */
    SEM_OPT_INNER_ITERATION = 8, /* FP32 inner MINRES iteration for Res: 1 (default) one grid
                                    barrier per iteration (operator product carried by
                                    recurrence), 0 the two-barrier form of the FP64 solver */
    SEM_OPT_REFINE_TOL_SCALE = 9, /* mixed mode stops at |r| < s (tol |r0| + tol), s in (0,1],
                                    default 1 (the reference's test on the true residual) */
    SEM_OPT_ADAPTIVE_INNER = 12, /* mixed mode: 1 (default) a sweep's inner tolerance is relaxed
                                    to what the outer test still needs (x 0.3), 0 always
                                    SEM_OPT_INNER_TOL */
    SEM_OPT_LEARNED_STEP = 15,   /* SEM_GUESS_LEARNED: 0 (default) move from the base guess along
                                    the predicted correction by the step that minimises the
                                    residual (FP32 apply of the correction against the base
                                    guess's FP64 residual); 1 take the whole predicted
                                    correction (the MINRES solve removes its high-frequency
                                    error quickly), unless its residual is not finite or more
                                    than 10x the base's */
    SEM_OPT_PROJECT = 14,        /* mixed mode with SEM_GUESS_EXTRAPOLATE / _LEARNED, SDIRK
                                    drivers: K in 1..24 replaces the extrapolation by the
                                    projection onto the last K stage solutions (the guess
                                    sum c_j z_j minimising |b - sum c_j b_j|, P. F. Fischer's
                                    method for successive right-hand sides; the learned
                                    correction then starts from it); 0 (default) off */
    SEM_OPT_RESIDENT = 13,       /* mixed mode, Res with SEM_PRECOND_FDM: 1 (default) keep the
                                    FP32 inner solve's vectors on chip (shared memory and
                                    registers; only element-ring copies are exchanged through
                                    global memory) when each SM's share of the mesh fits
                                    (p = 4, 6, 8, 10; up to 31 elements per SM at p = 8);
                                    0 always the staged kernel.  Same FP64 stopping test */
    SEM_OPT_EXTRAP_ORDER = 11,   /* stage guess of SEM_GUESS_EXTRAPOLATE / _LEARNED: 1 (default)
                                    linear 2 z1 - z2, 2 quadratic 3 z1 - 3 z2 + z3 once three
                                    previous steps exist */
    SEM_OPT_APPLY_PIPELINE = 10  /* FP32 standalone apply: 1 (default) bulk-copy pipelined element
                                    kernel when the input fields are 16-byte aligned, 0 the
                                    one-pass kernel; same results bit for bit.  2: the pipelined
                                    kernel computing the geometric factors from each element's
                                    corners instead of reading them (5 words per node moved
                                    instead of 9; FP32 rounding of the factors differs from
                                    the stored ones, within FP32 accuracy).  A pipelined
                                    apply whose bounded wait expired is reported as
                                    SEM_ERR_DEVICE_WAIT by the next sem_dot, solver or
                                    driver call */
};
enum { SEM_PREC_FP64 = 0, SEM_PREC_MIXED = 1 };
enum { SEM_PRECOND_NONE = 0, SEM_PRECOND_DIAG = 1, SEM_PRECOND_FDM = 2 };
enum { SEM_GUESS_ZERO = 0, SEM_GUESS_EXTRAPOLATE = 1, SEM_GUESS_LEARNED = 2 };

typedef struct sem_ctx sem_ctx;

/* include/solver_base.hpp:6-12 (solver_results<double>) */
typedef struct {
    int success;
    int n_iter;
    double residual;
} sem_solver_results;

/* include/ode_base.hpp:6-13 (solver_opts<double>) */
typedef struct {
    int max_iter;
    double tol;
    double dt;
    int verbose;
} sem_solver_opts;

typedef struct {
    int p, N;
    int n_elements, n_nodes, n_edges;
    int n_interior_edges, n_boundary_edges, n_boundary_nodes;
    long long n_local;      /* E*N*N */
    long long dof;          /* include/openmp_impl/Mesh.hpp:84-87 */
} sem_mesh_info;

typedef struct {
    long long krylov_iterations;    /* total MINRES/PCG iterations since creation */
    long long fp64_applies;         /* operator applies done in FP64 */
    long long fp32_applies;         /* operator applies done in FP32 */
    int last_step_stages;           /* stages in the last time step */
    int last_stage_iters[8];        /* Krylov iterations (inner, summed over sweeps) per stage */
    int last_stage_sweeps[8];       /* FP64 refinement sweeps per stage (1 in FP64 mode) */
    double last_error_estimate;     /* SDIRK4 5-stage embedded estimate (schrodinger.hpp:262-263) */
    int steps_taken;                /* steps of the last driver call */
    long long kernel_launches;      /* kernels this library launched since creation */
    long long solver_launches;      /* persistent solver launches since creation */
    double solver_kernel_ms;        /* their summed device time (SEM_OPT_PROFILE only) */
    long long solver_iterations_fp64; /* Krylov iterations run in FP64 */
    long long solver_iterations_fp32; /* Krylov iterations run in FP32 */
    long long learned_guesses;      /* stage guesses the learned model proposed */
    long long learned_accepted;     /* ... and that lowered the extrapolation's residual */
    double last_guess_residual_ratio; /* |r(guess used)| / |r(extrapolated)| of the last such stage */
    double last_guess_theta;        /* step taken along the predicted correction (1: as predicted) */
    double learned_ratio_sum;       /* sum of |r(guess used)| / |r(extrapolated)| over learned guesses */
    long long resident_launches;    /* persistent solver launches with the on-chip inner solve
                                       (SEM_OPT_RESIDENT) */
    long long projected_guesses;    /* stage guesses from the projection (SEM_OPT_PROJECT) */
    double last_projection_ratio;   /* |b - sum c_j b_j| / |b| of the last one */
    double projection_ratio_sum;    /* sum of that ratio over all projected guesses */
} sem_stats;

/* after each accepted step; nonzero return stops the time loop
 * (include/openmp_impl/schrodinger.hpp:116-118).  psi_re/psi_im point to
 * the caller's own buffers (host or device, as passed in), which already
 * hold the state after the step. */
typedef int (*sem_step_callback)(void* user, int step, const double* psi_re, const double* psi_im);

/* ---------------------------------------------------------------- misc */
int sem_version(void);
const char* sem_status_string(int status);
/* last error message of the calling thread ("" if none) */
const char* sem_last_error(void);

/* ---------------------------------------------------------------- mesh */

/* load_mesh<Mesh>(p, folder) + Mesh::compute_metrics()
 * (include/load_mesh.hpp:76-209, include/openmp_impl/Mesh.hpp:70-75) from
 * in-memory arrays: coords = n_nodes (x,y) pairs, elements = n_elements x 4
 * counter-clockwise corner ids.  1 <= p <= 16. */
int sem_ctx_create(sem_ctx** ctx, int p, int n_nodes, const double* coords,
                   int n_elements, const int* elements, unsigned flags);
/* the same from the reference's mesh folder (info.txt, coordinates.txt,
 * elements.txt; include/load_mesh.hpp:90-144) */
int sem_ctx_load(sem_ctx** ctx, int p, const char* folder, unsigned flags);
int sem_ctx_destroy(sem_ctx* ctx);
int sem_ctx_get_info(const sem_ctx* ctx, sem_mesh_info* info);
/* bind the context to a cudaStream_t (NULL = legacy default stream) */
int sem_ctx_set_stream(sem_ctx* ctx, void* cuda_stream);
int sem_ctx_set_option(sem_ctx* ctx, int option, double value);
int sem_ctx_get_stats(const sem_ctx* ctx, sem_stats* stats);
/* quad_rule (include/gauss_lobatto.hpp:27-32) and Mesh::D
 * (include/load_mesh.hpp:83): x, w hold N values, D N*N column-major.
 * Host pointers; any may be NULL. */
int sem_ctx_get_quadrature(const sem_ctx* ctx, double* x, double* w, double* D);
/* Quad::J, A, B, C of every element (include/Quad.hpp:17-20) as fields.
 * Host pointers; any may be NULL. */
int sem_ctx_get_metrics(const sem_ctx* ctx, double* J, double* A, double* B, double* C);
/* Quad::from_local_coo (include/Quad.hpp:57-62) at every element-local node.
 * Host pointers. */
int sem_ctx_get_node_coords(const sem_ctx* ctx, double* x, double* y);

/* ---------------------------------------------- gather-scatter (device) */

/* schro_omp::unmask (include/openmp_impl/unmask.hpp:43-55), in place */
int sem_unmask(sem_ctx* ctx, double* a);
/* schro_omp::global_sum (include/openmp_impl/global_sum.hpp:65-77), in place */
int sem_global_sum(sem_ctx* ctx, double* a);
/* schro_omp::mask (include/openmp_impl/mask.hpp:16-28), in place */
int sem_mask(sem_ctx* ctx, double* a);
/* schro_omp::dot (include/openmp_impl/dot.hpp:11-61); result to host */
int sem_dot(sem_ctx* ctx, const double* a, const double* b, double* result);
/* out = a*x + b*y over n values (y may be NULL, then out = a*x): the
 * element-wise algebra of the reference's expression templates
 * (include/Op.hpp:9-37, include/openmp_impl/solution_wrapper.hpp:150-185) */
int sem_vec_axpby(sem_ctx* ctx, long long n, double a, const double* x, double b,
                  const double* y, double* out);

/* ---------------------------------------------------- operators (device) */

/* schro_omp::gproj (include/openmp_impl/galerkin.hpp:42-57) */
int sem_gproj(sem_ctx* ctx, const double* u, double* out);
/* galerkin_op of glaplace: the Poisson operator
 * (include/openmp_impl/poisson.hpp:31-47, include/glaplace.hpp:16-28) */
int sem_apply_laplace(sem_ctx* ctx, const double* u, double* out);
/* Helmholtz operator (include/openmp_impl/helmholtz.hpp:32-52) */
int sem_apply_helmholtz(sem_ctx* ctx, const double* c, const double* u, double* out);
/* Schroedinger Res closure [M u + a L v ; a L u - M v], L = K + M_V
 * (include/openmp_impl/schrodinger.hpp:344-366) */
int sem_apply_schro_res(sem_ctx* ctx, const double* V, double alpha,
                        const double* q_re, const double* q_im, double* out_re, double* out_im);
/* Schroedinger f closure [-L v ; -L u] (include/openmp_impl/schrodinger.hpp:322-342) */
int sem_apply_schro_f(sem_ctx* ctx, const double* V,
                      const double* q_re, const double* q_im, double* out_re, double* out_im);
/* FP32 storage and arithmetic variant of sem_apply_schro_res (the operator
 * the FP32 inner solver applies; no reference counterpart in float) */
int sem_apply_schro_res_f32(sem_ctx* ctx, const float* V, float alpha,
                            const float* q_re, const float* q_im, float* out_re, float* out_im);

/* No counterpart in the reference.  The same operator as
 * sem_apply_schro_res for callers that must not allocate device memory:
 * code whose device memory is owned and budgeted by a host framework or pool
 * allocator, and latency-critical loops where the implicit synchronisation of
 * cudaMalloc/cudaFree is not acceptable.  Its element-local intermediate
 * lives in a static device array of 2^20 doubles (8 MiB, held by every GPU
 * that loads the library until exit) instead of a library allocation, so
 * the call allocates nothing.  Requires 2*E*N*N <= 1048576, otherwise it
 * returns SEM_ERR_UNSUPPORTED.  The first call on each device looks up the
 * array's device address; make that first call before any stream capture.
 * The context's device must be current (else SEM_ERR_ARG).  Outputs may
 * alias the inputs (in place).  All calls share the array: calls whose
 * kernels overlap on the GPU (other streams, other contexts) race on it.
 * Device pointers. */
int sem_apply_schro_res_noalloc(sem_ctx* ctx, const double* V, double alpha,
                                const double* q_re, const double* q_im,
                                double* out_re, double* out_im);

/* --------------------------------------------- Krylov solvers (device) */

/* minres (include/minres.hpp:19-107) on the Schroedinger Res operator with
 * the identity preconditioner, as schrodinger.hpp:97,223,380 call it.
 * x in/out; x_is_zero != 0 promises x == 0 on entry (skips A(x)). */
int sem_minres_schro(sem_ctx* ctx, const double* V, double alpha,
                     double* x_re, double* x_im, const double* b_re, const double* b_im,
                     int maxit, double tol, int x_is_zero, sem_solver_results* res);
/* minres on the Helmholtz operator (include/openmp_impl/helmholtz.hpp:59) */
int sem_minres_helmholtz(sem_ctx* ctx, const double* c, double* x, const double* b,
                         int maxit, double tol, int x_is_zero, sem_solver_results* res);
/* pcg (include/pcg.hpp:59-97) on the Poisson operator
 * (include/openmp_impl/poisson.hpp:54) */
int sem_pcg_laplace(sem_ctx* ctx, double* x, const double* b,
                    int max_iter, double tol, int x_is_zero, sem_solver_results* res);

/* --------------------------------------------- drivers (host or device) */

/* schro_omp::poisson (include/openmp_impl/poisson.hpp:17-59) */
int sem_poisson(sem_ctx* ctx, double* u, const double* f, int max_iter, double tol,
                sem_solver_results* res);
/* schro_omp::helmholtz (include/openmp_impl/helmholtz.hpp:18-64) */
int sem_helmholtz(sem_ctx* ctx, double* u, const double* c, const double* f,
                  int max_iter, double tol, sem_solver_results* res);
/* Poisson and Helmholtz with boundary data, no counterpart in the reference
 * (whose masks zero every boundary copy: include/mask_side.hpp:28-30).
 *  - Dirichlet context (default): u = g on the boundary.  g is an
 *    element-local field (E*N*N) of which the copies of boundary nodes are
 *    read.  By lifting: with u_D = g on those copies and 0 elsewhere, the
 *    masked system A u0 = gproj(f) - A u_D is solved (PCG / MINRES as
 *    sem_poisson / sem_helmholtz) and u = u0 + u_D.
 *  - SEM_FLAG_NEUMANN context: du/dn = g on the boundary.  g holds the
 *    outward normal derivative per element side node, E*4*N values: side s
 *    (0: j = 0, 1: i = N-1, 2: j = N-1, 3: i = 0), node k = 0..N-1 along the
 *    side (the element's i on sides 0 and 2, its j on sides 1 and 3); only
 *    boundary sides are read (a domain corner takes each side's own value).
 *    The boundary integral of the weak form, sum over boundary sides of
 *    w_k (L/2) g_k (GLL quadrature on the straight side of length L), is
 *    added to gproj(f).  Poisson with only Neumann data is singular; use
 *    Helmholtz with c > 0 there.
 * u in: initial guess (its boundary copies are ignored for Dirichlet data);
 * out: the solution at every copy (continuous format).  Host or device
 * pointers. */
int sem_poisson_bc(sem_ctx* ctx, double* u, const double* f, const double* g, int max_iter,
                   double tol, sem_solver_results* res);
int sem_helmholtz_bc(sem_ctx* ctx, double* u, const double* c, const double* f, const double* g,
                     int max_iter, double tol, sem_solver_results* res);
/* schro_omp::schrodinger_bdf2 (include/openmp_impl/schrodinger.hpp:22-128) */
int sem_schrodinger_bdf2(sem_ctx* ctx, double* psi_re, double* psi_im, const double* V,
                         double T, const sem_solver_opts* opts,
                         sem_step_callback cb, void* user, int* success);
/* schro_omp::schrodinger_dirk4s5 (include/openmp_impl/schrodinger.hpp:138-285) */
int sem_schrodinger_dirk4s5(sem_ctx* ctx, double* psi_re, double* psi_im, const double* V,
                            double T, const sem_solver_opts* opts,
                            sem_step_callback cb, void* user, int* success);
/* schro_omp::schrodinger_dirk4s3 (include/openmp_impl/schrodinger.hpp:294-423) */
int sem_schrodinger_dirk4s3(sem_ctx* ctx, double* psi_re, double* psi_im, const double* V,
                            double T, const sem_solver_opts* opts,
                            sem_step_callback cb, void* user, int* success);

/* No counterpart in the reference (its 5-stage driver, schrodinger.hpp:138-285,
 * only prints the embedded error estimate of :262-263).  Adaptive SDIRK4
 * 5-stage: a step is accepted when |sum_l e_l z_l| / |psi_0| <= err_tol, the
 * next dt is dt * clamp(0.9 (err_tol/err)^(1/4), 0.2, 2) (at most 0.9 after
 * a rejection), the last step lands on T.  opts->dt is the first trial step.
 * dts (host, may be NULL) receives the accepted steps' dt, up to
 * dts_capacity of them (the sequence replays the fixed-step reference).  In
 * mixed precision with a stage guess other than SEM_GUESS_ZERO a stage starts
 * from the last accepted step's stage scaled by the dt ratio; with
 * SEM_GUESS_LEARNED and a network set, the network corrects that guess as in
 * the fixed-step drivers, and sem_ctx_record collects training rows from
 * these stages too. */
int sem_schrodinger_dirk4s5_adaptive(sem_ctx* ctx, double* psi_re, double* psi_im, const double* V,
                                     double T, const sem_solver_opts* opts, double err_tol,
                                     double* dts, int dts_capacity, int* n_accepted, int* n_rejected,
                                     sem_step_callback cb, void* user, int* success);

/* ------------------------------------------- learned stage guess (device)
 * No counterpart in the reference (its stage solves start from zero,
 * schrodinger.hpp:222,379).  A per-element network predicts the error of the
 * extrapolated stage guess 2 z^{n-1} - z^{n-2} from that guess's residual.
 * Rows are elements: input 4 N^2 BF16 features [r_re/rho, r_im/rho,
 * alpha V, mass/alpha] with rho the element's RMS residual; output 2 N^2
 * FP32 values, the correction (z - z_guess) mbar/rho with mbar the element's
 * mean lumped mass.  Network: ReLU MLP d_in -> H -> H -> d_out,
 * BF16 tensor-core GEMMs with FP32 accumulation, FP32 master weights, Adam.
 * Weights W are [in][out] row-major FP32. */
typedef struct sem_learner sem_learner;
int sem_learner_create(sem_learner** learner, int d_in, int hidden, int d_out,
                       unsigned long long seed);
int sem_learner_destroy(sem_learner* learner);
int sem_learner_shape(const sem_learner* learner, int* d_in, int* hidden, int* d_out);
int sem_learner_set_stream(sem_learner* learner, void* cuda_stream);
/* host copies of layer l (0..2) weights [in][out] and biases [out] */
int sem_learner_get_params(sem_learner* learner, int l, float* W, float* b);
int sem_learner_set_params(sem_learner* learner, int l, const float* W, const float* b);
/* out (device FP32, rows x d_out) = network(x), x device BF16 rows x d_in */
int sem_learner_forward(sem_learner* learner, int rows, const void* x_bf16, float* out);
/* one batch: loss = mean((net(x) - target)^2) to *loss (host, may be NULL);
 * gradients kept for sem_learner_get_grads; lr > 0 also takes an Adam step */
int sem_learner_train_step(sem_learner* learner, int rows, const void* x_bf16,
                           const float* target, float lr, double* loss);
int sem_learner_get_grads(sem_learner* learner, int l, float* gW, float* gb);
/* Adam over `epochs` shuffled passes of minibatches of `batch` rows of a
 * device dataset (X BF16 rows x d_in, T FP32 rows x d_out) */
int sem_learner_fit(sem_learner* learner, const void* X, const float* T, long long rows,
                    int epochs, int batch, float lr, unsigned long long seed, double* final_loss);
/* C (M x N FP32) = A (M x K BF16) B (K x N BF16), row-major device arrays,
 * the network's tensor-core GEMM */
int sem_gemm_bf16(int M, int N, int K, const void* A, const void* B, float* C, void* cuda_stream);
/* (no counterpart in the reference) Tensor-core instruction path of every
 * GEMM of the learned-guess network and of sem_gemm_bf16, process-wide:
 * 1 (default) tcgen05.mma with the accumulator in tensor memory (M = 128
 * per CTA, BF16 operands from shared memory, FP32 accumulation), and the
 * network's inference pass (sem_learner_forward) fused into one launch that
 * chains the three layers through tensor and shared memory when the hidden
 * and output widths are at most 256; 2 the same tcgen05 GEMMs one layer per
 * launch; 0 the warp-level mma.sync m16n8k16 kernel.  All compute in
 * BF16 x BF16 -> FP32 with BF16 hidden activations. */
int sem_gemm_set_path(int path);
/* (no counterpart in the reference) *expired = 1 when a bounded wait of a
 * tcgen05 GEMM ever ran out in this process (its output tile was then left
 * unwritten); 0 otherwise */
int sem_gemm_check_error(int* expired);
/* network used by the SDIRK drivers when SEM_OPT_STAGE_GUESS is
 * SEM_GUESS_LEARNED in mixed precision (NULL: extrapolation only).  The
 * caller keeps ownership.  Every proposed guess is checked in FP64: the
 * driver moves from the extrapolation along the predicted correction by the
 * step that minimises the residual norm (the extrapolation itself when no
 * positive step lowers it). */
int sem_ctx_set_learner(sem_ctx* ctx, sem_learner* learner);
/* record training rows from the SDIRK drivers' stage solves (mixed precision,
 * SEM_GUESS_EXTRAPOLATE or _LEARNED, from the third step on; in the adaptive
 * driver from the second accepted step on) into a device
 * dataset of capacity_rows rows; 0 stops recording.  Resets the dataset. */
int sem_ctx_record(sem_ctx* ctx, long long capacity_rows);
/* the recorded dataset: device pointers X (BF16 rows x d_in), T (FP32 rows x
 * d_out), rows recorded, d_in = 4 N^2, d_out = 2 N^2 */
int sem_ctx_dataset(sem_ctx* ctx, void** X, float** T, long long* rows, int* d_in, int* d_out);

/* ------------------------------------------------- batched ensembles (device)
 * No counterpart in the reference (its drivers step one mesh).  Many
 * independent instances -- each with its own mesh (p = 2..8), potential and
 * state -- advanced together by schro_omp::schrodinger_bdf2
 * (include/openmp_impl/schrodinger.hpp:22-128) with the mixed-precision
 * stage solve (FP32 inner MINRES, FP64 refinement on the true residual;
 * SEM_PRECOND_FDM by default).  One persistent launch per time step serves
 * all instances (a block per instance, largest first, block-local barriers
 * and reductions); the step is captured once as a CUDA graph and replayed.
 * The elements each block stages per pass are chosen per degree by a timing
 * sweep at creation (sem_batch_stats.kmax_of_p). */
typedef struct sem_batch sem_batch;
typedef struct {
    long long steps;              /* time steps run (all instances together) */
    long long instance_steps;     /* instance-steps */
    long long krylov_iterations;  /* FP32 inner iterations over all instances */
    long long graph_launches;     /* replays of the captured step */
    long long graphs_built;       /* step captures */
    double kernel_ms;             /* device time of the replayed steps */
    int kmax_of_p[17];            /* elements staged per pass, by degree p (0: absent) */
} sem_batch_stats;
/* instance i: degree p[i], n_nodes[i] corner coordinates coords[i] (x,y
 * pairs), n_elements[i] quads elements[i] (4 counter-clockwise corner ids) */
int sem_batch_create(sem_batch** batch, int n_instances, const int* p, const int* n_nodes,
                     const double* const* coords, const int* n_elements, const int* const* elements,
                     unsigned flags);
int sem_batch_destroy(sem_batch* batch);
int sem_batch_set_stream(sem_batch* batch, void* cuda_stream);
/* SEM_OPT_INNER_TOL, SEM_OPT_MAX_REFINE, SEM_OPT_REFINE_TOL_SCALE,
 * SEM_OPT_PRECOND (NONE or FDM); SEM_OPT_SOLVE_PRECISION only MIXED */
int sem_batch_set_option(sem_batch* batch, int option, double value);
int sem_batch_get_info(const sem_batch* batch, int instance, sem_mesh_info* info);
int sem_batch_get_stats(const sem_batch* batch, sem_batch_stats* stats);
/* after a driver call: steps taken, whether the instance stopped on a failed
 * solve, and its inner iterations */
int sem_batch_get_instance(const sem_batch* batch, int instance, int* steps, int* stopped,
                           long long* iterations);
/* schrodinger_bdf2 for every instance at once: per-instance field pointers
 * (host or device), in/out state; success[i] as the reference's return */
int sem_batch_schrodinger_bdf2(sem_batch* batch, double* const* psi_re, double* const* psi_im,
                               const double* const* V, double T, const sem_solver_opts* opts,
                               int* success);

#ifdef __cplusplus
}
#endif
#endif /* SEM_GB300_H */
