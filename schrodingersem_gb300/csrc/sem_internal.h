// Internal declarations shared by the host side (sem_host.cu) and the
// per-degree kernel instantiation units (sem_inst.cu).  Not installed.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace semgb {

constexpr int MIN_N = 2;   // p = 1
constexpr int MAX_N = 17;  // p = 16
constexpr int CORNER_NB_MAX = 8;  // copies per corner node held in DevMesh::corner_nb / node_nb
static_assert(CORNER_NB_MAX % 4 == 0, "node_nb rows are read as int4");

// Element-local operator kinds (the closures of the reference's drivers).
enum OpKind : int {
    OP_LAPLACE = 0,  // glaplace                         (glaplace.hpp:16-28)
    OP_HELM = 1,     // glaplace + (W (u%c) W) % J      (helmholtz.hpp:44-45)
    OP_MASS = 2,     // (W u W) % J                      (galerkin.hpp:51)
    OP_RES = 3,      // [M u + a L v ; a L u - M v]      (schrodinger.hpp:353-360)
    OP_F = 4         // [-L v ; -L u]                    (schrodinger.hpp:331-336)
};

// Assembly modes of the direct-stiffness sum.
enum DssMode : int {
    DSS_SUM = 0,   // global_sum: shared interior nodes get the sum at every copy, boundary untouched
    DSS_MASK = 1,  // global_sum then mask: sum at the owner copy, zero elsewhere and on the boundary
    DSS_CONT = 2   // sum at every copy, zero on the boundary (the solvers' continuous format)
};

// Per-element topology bits in DevMesh::flags.
//  bits 0-3   side s owned by this element (it is Edge::elements[0])
//  bits 4-7   side s on the boundary
//  bits 8-11  corner c owned (first of CornerNode::connected_elements)
//  bits 12-15 corner c on the (Dirichlet) boundary
//  bits 16-19 side s on a Neumann boundary: owned, no partner copy (a Neumann
//             context leaves the boundary bits clear; its boundary corners
//             assemble over their copies like interior corners)
// Sides s = 0..3 are the reference's sides 1..4: j=0, i=N-1, j=N-1, i=0.
// Corners c = 0..3 are (0,0), (N-1,0), (N-1,N-1), (0,N-1).

struct DevMesh {
    int N = 0, E = 0, n_nodes = 0;
    long long n = 0;  // E*N*N
    const int* flags = nullptr;
    const int* side_base = nullptr;  // [E*4] neighbour flat index at k = 0 (valid for interior sides)
    const int* side_step = nullptr;  // [E*4] neighbour flat-index step per k
    const int* corner_src = nullptr; // [E*4] flat index of the corner's owner copy
    const int* corner_node = nullptr;// [E*4] corner node id
    const int* node_ptr = nullptr;   // [n_nodes+1] CSR over copies of each corner node
    const int* node_flat = nullptr;  // flat indices of the copies, element order
    const double* kdiag = nullptr;   // diagonal of the assembled stiffness (continuous format)
    const double* mdiag = nullptr;   // assembled lumped mass w_i w_j J (continuous format)
    const double* D64 = nullptr;     // D row-major: D(i,k) at [i*N+k]
    const float* D32 = nullptr;
    // premultiplied factors w_i w_j {A, B, C, J}
    const double *g11 = nullptr, *g12 = nullptr, *g22 = nullptr, *mass = nullptr;
    const float *g11f = nullptr, *g12f = nullptr, *g22f = nullptr, *massf = nullptr;
    // element fast-diagonalisation preconditioner: 1-D GLL generalised
    // eigenvectors S(i,k) at [i*N+k] (K s = lambda W s, S^T W S = I), their
    // eigenvalues, and per element {ax ay, ay/ax, ax/ay, 0} of the element's
    // rectangle approximation (half widths ax, ay)
    const double* fdmS64 = nullptr;
    const float* fdmS32 = nullptr;
    const double* fdmL64 = nullptr;
    const float* fdmL32 = nullptr;
    const float4* fdm_el = nullptr;
    // ring tables: ring_src[e*4(N-1) + r] = flat index of the owner copy for
    // the non-owner, non-boundary ring copy r of element e (ring order: j=0
    // side, i=N-1 side, j=N-1 side reversed, i=0 side reversed), else -1;
    // edge_pairs = (owner, other) copies of every interior-side node (corners
    // excluded); bnd_flat = copies on boundary sides (corners excluded);
    // node_bnd = corner node on the boundary
    const int* ring_src = nullptr;
    // corner copies of every element corner (4 per element, CORNER_NB_MAX
    // entries each): the flat indices of all copies of the corner node in
    // CSR order, -1 padded, first entry -2 when the node has more copies;
    // corner_cnt4[e] packs the four corners' copy counts, 8 bits each
    const int* corner_nb = nullptr;
    const int* corner_cnt4 = nullptr;
    // the same lists per corner node (n_nodes rows of CORNER_NB_MAX)
    const int* node_nb = nullptr;
    const int2* edge_pairs = nullptr;
    const int* bnd_flat = nullptr;
    const char* node_bnd = nullptr;
    long long n_pairs = 0, n_bnd = 0;
    // pipelined FP32 apply: side pairs with both copies inside one batch of
    // bulk_K elements are summed by the apply kernel itself; edge_pairs lists
    // the other pairs first (n_pairs_x of them).  bulk_pair_ptr[b] ..
    // bulk_pair_ptr[b+1] index bulk_pairs of batch b, each packing the batch-
    // local flat offsets (owner << 16 | other)
    long long n_pairs_x = 0;
    int bulk_K = 0;
    const int* bulk_pair_ptr = nullptr;
    const int* bulk_pairs = nullptr;
    int* dev_err = nullptr;  // set by a kernel whose bounded wait expired (pipelined apply)
    const double* Dh = nullptr;  // host copy of D, row-major (launchers that pass D by value)
    // on-the-fly geometry of the FP32 Res apply: per element {x1-x0, x2-x3,
    // x3-x0, x2-x1, y1-y0, y2-y3, y3-y0, y2-y1} (FP32), the host LGL nodes and
    // weights, and the metric convention (1: SEM_FLAG_METRIC_CORRECTED)
    const float* geo32 = nullptr;
    const double* zh = nullptr;
    const double* wh = nullptr;
    int corrected = 0;
};

// Grid barrier and error state of a persistent (cooperative) kernel.
struct GridSync {
    unsigned int count;
    unsigned int gen;
    int err;   // nonzero: a wait hit its limit
    int pad;
};

// Device-side result of a persistent solve.
struct SolveOut {
    int success;
    int n_iter;
    double residual;
    int status;      // 0 or SEM_ERR_DEVICE_WAIT
    int inner_iters; // mixed mode: total FP32 iterations
    int sweeps;      // mixed mode: refinement sweeps
    int pad;
};

template <typename T>
struct KrylovWork {
    T* L[3];        // Lanczos vectors (NC planes each)
    T* W[3];        // MINRES direction vectors / PCG p, r
    T* Y[2];        // element-local operator output
    double* partials;  // [2 slots][grid][4]
    T* AZ;          // single-barrier MINRES: assembled A z_i (continuous format)
    T* Y3;          // single-barrier MINRES: y_i before the r2 correction
    T* Z[2];        // element preconditioner: z = P^-1 r of the last two iterations
};

struct SolveArgs {
    int op;          // OP_RES, OP_HELM, OP_LAPLACE
    int nc;          // 1 or 2 planes
    const void* pot; // V or c field (same precision as T), may be null for LAPLACE
    double alpha;
    const void* b[2]; // right-hand side planes (masked format)
    void* x[2];       // solution planes, in/out
    int maxit;
    double tol;
    int x_is_zero;
    int kmax;         // elements staged per pass (solver_plan)
    int rel_to_b;     // mixed solver: stop on |r| < tol |b| + tol instead of tol |r_0| + tol
                      // (the same test when x_0 = 0; used with warm starts)
    long long timeout_ns;
    GridSync* sync;
    SolveOut* out;
};

// Mixed-precision refinement: FP64 true residual and solution, FP32 inner
// MINRES (see k_minres_mixed).
struct MixedArgs {
    double inner_tol;
    int max_sweeps;
    int inner_maxit;
    double* r64[2];      // FP64 residual planes
    double* Y64[2];      // FP64 element-local output planes
    float* x32[2];       // FP32 correction planes
    const float* pot32;  // FP32 copy of the potential (V or c)
    const float* pinv32; // diagonal preconditioner P^-1 (continuous format), or null
    int fdm;             // element fast-diagonalisation preconditioner (Res only; uses KrylovWork::Z)
    int fused;           // inner solve with the single-barrier MINRES iteration (Res only)
    double outer_scale;  // refinement stops at |r| < outer_scale * (tol |r0| + tol)
    int adaptive;        // inner tolerance of a sweep no tighter than the outer test needs
};

// ---- launchers, one explicit instantiation per N in sem_inst.cu -------------
template <int N>
cudaError_t launch_apply(const DevMesh& m, int op, bool fp32, const void* pot, double alpha,
                         const void* in0, const void* in1, void* y0, void* y1, bool gather,
                         cudaStream_t st);
// the FP32 Res operator through the bulk-copy pipeline (k_apply_bulk); every
// field pointer 16-byte aligned (FP64 applies are FP64-pipe bound and use
// the one-pass kernel).  pair_asm: the kernel also sums the side pairs inside
// its batches (the masked output then needs launch_ring with cross_only).
// geo: the geometric factors computed on the fly from the element corners
// (FP32 Res; DevMesh::geo32), not read from the stored planes
template <int N>
cudaError_t launch_apply_bulk(const DevMesh& m, int op, bool fp32, const void* pot, double alpha, const void* in0,
                              const void* in1, void* y0, void* y1, bool gather, bool pair_asm, bool geo,
                              long long timeout_ns, cudaStream_t st);
template <int N>
cudaError_t launch_dss(const DevMesh& m, bool fp32, int mode, double scale, const void* y,
                       void* out, cudaStream_t st);
// in-place assembly of element-local values touching only element rings
// (k_ring); equals launch_dss with scale 1 into a separate output
template <int N>
// cross_only: only the side pairs that cross batches of the pipelined apply
// (the apply kernel summed the others)
cudaError_t launch_ring(const DevMesh& m, bool fp32, int mode, void* a0, void* a1, bool cross_only,
                        cudaStream_t st);
template <int N>
cudaError_t launch_unmask(const DevMesh& m, bool fp32, void* a, cudaStream_t st);
template <int N>
cudaError_t launch_mask(const DevMesh& m, bool fp32, void* a, cudaStream_t st);
// weighted dot: partial sums per block into part[grid], returns grid used
template <int N>
cudaError_t launch_dot(const DevMesh& m, const double* a, const double* b, double* part,
                       int max_blocks, int* blocks_used, cudaStream_t st);
// (a.a, a.b, b.b) over both planes of two-plane vectors, 3 partials per block
template <int N>
cudaError_t launch_dot3(const DevMesh& m, const double* a, const double* b, double* part, int max_blocks,
                        int* blocks_used, cudaStream_t st);
// the same with an FP32 second vector (FP64 sums)
template <int N>
cudaError_t launch_dot3_f32(const DevMesh& m, const double* a, const float* b, double* part, int max_blocks,
                            int* blocks_used, cudaStream_t st);
// out[n] = gather(p + sum_l c[l] z_l) for every node (unmask semantics); then
// optional f-apply: y = L-closure of the combination.
struct ZList {
    int nz;
    const double* z[8];  // two-plane vectors (plane stride n)
    double c[8];
};
template <int N>
cudaError_t launch_combo_f(const DevMesh& m, const double* V, const double* p, const ZList& zl,
                           double* y, cudaStream_t st);
// p_out = unmask(p_in + sum_l c[l] z_l), both planes
template <int N>
cudaError_t launch_update(const DevMesh& m, const double* p_in, const ZList& zl, double* p_out,
                          cudaStream_t st);
// per-element kernels of the learned stage guess (see k_features)
enum LearnWhat : int { LEARN_RESID = 0, LEARN_FEATURES = 1, LEARN_TARGETS = 2, LEARN_CORRECT = 3 };
struct LearnArgs {
    int what;
    const double* b;      // RESID: right-hand side (masked), 2 planes
    const double* Y;      // RESID: element-local operator output of the guess, 2 planes
    double* r;            // RESID out / FEATURES in: residual (continuous), 2 planes
    const double* V;      // FEATURES: potential
    double alpha;         // FEATURES: stage coefficient
    double rho_floor;     // FEATURES: lower bound of the per-element residual scale
    void* x;              // FEATURES out: BF16 rows [E][4 N^2]
    float* sigma;         // FEATURES out / TARGETS, CORRECT in: per-element scale
    const double* z;      // TARGETS: converged stage solution
    const double* zg;     // TARGETS, CORRECT: the guess it started from
    float* t;             // TARGETS out: FP32 rows [E][2 N^2]
    const float* delta;   // CORRECT: predicted rows [E][2 N^2]
    double* zo;           // CORRECT out: corrected guess
};
template <int N>
cudaError_t launch_learn(const DevMesh& m, const LearnArgs& a, cudaStream_t st);
// persistent Krylov solvers (cooperative launch).  solver_plan picks the grid
// (at most one block per SM) and the per-pass staging capacity in elements;
// launch_solver runs MINRES (op OP_RES/OP_HELM), PCG (OP_LAPLACE) or, when
// mx is given, the mixed-precision refinement.  work points to a
// KrylovWork<double> (FP64 solvers) or KrylovWork<float> (mixed).
template <int N>
int solver_plan(int op, bool mixed, int E, int sms, size_t smem_budget, int* kmax, size_t* smem);
template <int N>
cudaError_t launch_solver(const DevMesh& m, const SolveArgs& a, const void* work, const MixedArgs* mx,
                          int grid, size_t smem, cudaStream_t st);
// mixed-precision refinement with the on-chip resident FP32 inner solve
// (Res operator, element preconditioner; sem_resident.cuh), instantiated for
// N = 5, 7, 9, 11.  resident_plan returns false when a block's share of the
// mesh does not fit on chip; then the staged kernel (launch_solver) is used.
// D32h / S32h: host FP32 copies of D and of the preconditioner basis S, both
// row-major.  slots: 2 * grid * RESIDENT_SLOT_STRIDE words; xa, xb: 2 n words
// each (the tagged ring exchange); all cleared before the launch.
constexpr int RESIDENT_SLOT_STRIDE = 16;  // one 128-byte line per block's all-reduce word
template <int N>
bool resident_plan(int E, int sms, size_t smem_budget, int* grid, int* st, int* kmax64, size_t* smem);
template <int N>
cudaError_t launch_resident(const DevMesh& m, const SolveArgs& a, const KrylovWork<float>& w, const MixedArgs& mx,
                            const float* D32h, const float* S32h, int st, unsigned long long* slots,
                            unsigned long long* xa, unsigned long long* xb, int grid, size_t smem,
                            cudaStream_t stream);

}  // namespace semgb

// ---- context accessors (defined in sem_host.cu) ------------------------------
struct sem_ctx;
namespace semgb {
const DevMesh& ctx_mesh(const sem_ctx* c);
cudaStream_t ctx_stream(const sem_ctx* c);
void ctx_count_launches(sem_ctx* c, long long k);
int ctx_device(const sem_ctx* c);     // ordinal of the device the context was created on
void ctx_count_fp64_apply(sem_ctx* c);  // one more FP64 operator apply in sem_stats
int ctx_fail(int code, const char* msg);  // records the message, returns code
}  // namespace semgb
// kernels launched by a network's forward passes so far (defined in sem_mlp.cu)
struct sem_learner;
long long learner_forward_launches(const sem_learner* L);

#define SEM_FOR_EACH_N(X) \
    X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16) X(17)
