// Host side of the GB300 spectral-element library: mesh setup (topology,
// LGL quadrature, metrics), device buffers, dispatch over the polynomial
// degree, and every extern "C" entry point of include/sem_gb300.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "sem_gb300.h"
#include "sem_internal.h"
#include "sem_apply_bulk.cuh"

using namespace semgb;

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

static int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

#define SEM_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(SEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// the degrees with an on-chip resident inner solver (sem_resident.cu)
template <class F>
static bool dispatch_resident(int N, F&& f)
{
    switch (N) {
        case 5: f(std::integral_constant<int, 5>{}); return true;
        case 7: f(std::integral_constant<int, 7>{}); return true;
        case 9: f(std::integral_constant<int, 9>{}); return true;
        case 11: f(std::integral_constant<int, 11>{}); return true;
        default: return false;
    }
}

template <class F>
static cudaError_t dispatch_n(int N, F&& f)
{
    switch (N) {
#define SEM_CASE(NV) \
    case NV: return f(std::integral_constant<int, NV>{});
        SEM_FOR_EACH_N(SEM_CASE)
#undef SEM_CASE
        default: return cudaErrorInvalidValue;
    }
}

// ------------------------------------------------------------ small kernels
__global__ void k_axpby(long long n, double a, const double* __restrict__ x, double b,
                        const double* __restrict__ y, double* __restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = a * x[i];
        out[i] = y ? v + b * y[i] : v;
    }
}

__global__ void k_lincomb(long long n, ZList zl, double* __restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        double acc = zl.c[0] * zl.z[0][i];
        for (int l = 1; l < zl.nz; ++l) acc = acc + zl.c[l] * zl.z[l][i];
        out[i] = acc;
    }
}

__global__ void k_to_f32(long long n, const double* __restrict__ a, float* __restrict__ b)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// Projection stage guess (no counterpart in the reference): the previous
// stage solutions z_j of the same operator and their right-hand sides b_j.
constexpr int PROJ_MAX = 24;
struct PtrList {
    int nz;
    const double* z[PROJ_MAX + 1];
    double c[PROJ_MAX + 1];
};

// per-block partial sums of b.b_j (j < L.nz) and b.b, laid out
// part[blk * (PROJ_MAX + 1) + j] (b.b at j = PROJ_MAX); fixed order.  On
// masked vectors the plain sum equals the reference's unique-DOF dot.
__global__ void __launch_bounds__(256) k_multidot(long long n, const double* __restrict__ b, PtrList L,
                                                  double* __restrict__ part)
{
    double acc[PROJ_MAX + 1];
#pragma unroll
    for (int l = 0; l <= PROJ_MAX; ++l) acc[l] = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double bv = b[i];
        acc[PROJ_MAX] = fma(bv, bv, acc[PROJ_MAX]);
#pragma unroll
        for (int l = 0; l < PROJ_MAX; ++l)
            if (l < L.nz) acc[l] = fma(bv, __ldg(L.z[l] + i), acc[l]);
    }
    __shared__ double red[8][PROJ_MAX + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int l = 0; l <= PROJ_MAX; ++l) {
        double v = acc[l];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[wid][l] = v;
    }
    __syncthreads();
    if (threadIdx.x <= PROJ_MAX) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
        part[(size_t)blockIdx.x * (PROJ_MAX + 1) + threadIdx.x] = v;
    }
}

// out = sum_l c_l z_l over up to PROJ_MAX + 1 vectors
__global__ void k_lincomb_n(long long n, PtrList L, double* __restrict__ out)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        double acc = 0.0;
#pragma unroll
        for (int l = 0; l <= PROJ_MAX; ++l)
            if (l < L.nz) acc = fma(L.c[l], __ldg(L.z[l] + i), acc);
        out[i] = acc;
    }
}

// Step length of the learned guess from launch_dot3_f32's partials of
// (r_ext.r_ext, r_ext.Ad, Ad.Ad), summed in a fixed order: the step theta
// along d = z_l - z_ext minimising |r_ext - theta A d|, or the whole step
// when full_step and the prediction is finite and raises the residual at
// most tenfold (|r_l|^2 = |r_ext|^2 - 2 r_ext.Ad + |Ad|^2).
// st = (|r_ext|^2, theta, residual ratio, accepted 1/0).
__global__ void __launch_bounds__(256) k_learn_theta(const double* __restrict__ part, int used, int full_step,
                                                     double* __restrict__ st)
{
    __shared__ double red[3][256];
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < used; i += 256) {
        a += part[3 * i];
        b += part[3 * i + 1];
        c += part[3 * i + 2];
    }
    red[0][threadIdx.x] = a;
    red[1][threadIdx.x] = b;
    red[2][threadIdx.x] = c;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
#pragma unroll
            for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double n_ext = red[0][0], rad = red[1][0], den = red[2][0];
        double theta = den > 0 ? rad / den : 0.0;
        const double n_l = n_ext - 2.0 * rad + den;
        if (full_step && isfinite(n_l) && n_l <= 100.0 * n_ext) theta = 1.0;
        double ratio = 1.0, acc = 0.0;
        if (theta > 0 && n_ext > 0) {
            acc = 1.0;
            const double n_t = n_ext - 2.0 * theta * rad + theta * theta * den;  // |r_ext - theta A d|^2
            ratio = sqrt(fmax(0.0, n_t) / n_ext);
        }
        st[0] = n_ext;
        st[1] = theta;
        st[2] = ratio;
        st[3] = acc;
    }
}

// d = z_l - z_ext in FP32 (both planes)
__global__ void k_diff_f32(long long n, const double* __restrict__ zl, const double* __restrict__ zx,
                           float* __restrict__ d)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        d[i] = (float)(zl[i] - zx[i]);
}

// z = (1 - theta) z_ext + theta z_l when the step was accepted (st[3]);
// otherwise z keeps the base guess
__global__ void k_learn_step(long long n, const double* __restrict__ zx, const double* __restrict__ zl,
                             const double* __restrict__ st, double* __restrict__ z)
{
    if (st[3] == 0.0) return;
    const double th = st[1];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        z[i] = (1.0 - th) * zx[i] + th * zl[i];
}

static int grid_1d(long long n) { return (int)std::min<long long>((n + 255) / 256, 152 * 16); }

// dynamic shared memory a persistent solver block may use for staging
static const size_t kSolverSmemBudget = 160 * 1024;
// the resident inner solve may use all of an SM's shared memory (227 KB per
// block, less the kernel's static arrays)
static const size_t kResidentSmemBudget = 227 * 1024 - 512;

// Diagonal preconditioner P^-1 (continuous format).  Res = [M, aL; aL, -M]:
// P = diag(d, d), d = sqrt(m^2 + a^2 (k + m V)^2), the diagonal of |Res|
// when M and L are replaced by their diagonals.  Helmholtz K + M c:
// d = k + m |c|.  m, k: assembled mass and stiffness diagonals.
__global__ void k_prec(long long n, int op, double alpha, const double* __restrict__ mdiag,
                       const double* __restrict__ kdiag, const double* __restrict__ pot,
                       float* __restrict__ pinv)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double m = mdiag[i], k = kdiag[i];
        double d;
        if (op == OP_RES) {
            const double l = k + m * pot[i];
            d = sqrt(m * m + alpha * alpha * l * l);
        } else {
            d = k + m * fabs(pot[i]);
        }
        pinv[i] = (float)(1.0 / d);
    }
}

// --------------------------------------------------------------- quadrature
static double legendre(int n, double x)
{
    if (n == 0) return 1.0;
    double p0 = 1.0, p1 = x;
    for (int k = 1; k < n; ++k) {
        const double p2 = ((2.0 * k + 1.0) * x * p1 - k * p0) / (k + 1.0);
        p0 = p1;
        p1 = p2;
    }
    return p1;
}

// LGL nodes and weights of degree p (N = p+1 values).  For p <= 8 the
// reference's stated 15-digit nodes are used so the discretisation is the
// reference's own (include/gauss_lobatto.hpp:49-58).  For p > 8 the interior
// nodes, the roots of P_{p+1} - P_{p-1}, come from Newton's method started at
// the Chebyshev-Gauss-Lobatto points.  Weights 2/(p(p+1) P_p(x)^2)
// (include/gauss_lobatto.hpp:116-123).
static void lgl(int p, std::vector<double>& x, std::vector<double>& w)
{
    static const std::vector<std::vector<double>> tab = {
        {},
        {-1, 1},
        {-1, 0, 1},
        {-1, -0.447213595499958, 0.447213595499958, 1},
        {-1, -0.654653670707977, 0, 0.654653670707977, 1},
        {-1, -0.765055323929465, -0.285231516480645, 0.285231516480645, 0.765055323929465, 1},
        {-1, -0.830223896278567, -0.468848793470714, 0.0, 0.468848793470714, 0.830223896278567, 1},
        {-1, -0.871740148509607, -0.591700181433142, -0.209299217902479, 0.2092992179024789,
         0.591700181433142, 0.871740148509607, 1},
        {-1, -0.899757995411460, -0.677186279510738, -0.363117463826178, 0, 0.363117463826178,
         0.677186279510738, 0.899757995411460, 1}};
    x.assign(p + 1, 0.0);
    w.assign(p + 1, 0.0);
    if (p <= 8) {
        x = tab[p];
    } else {
        const int h = (p - 1) / 2;  // interior roots strictly below zero
        std::vector<double> neg(h);
        for (int k = 0; k < h; ++k) {
            double z = -std::cos(M_PI * (k + 1) / p);
            for (int it = 0; it < 100; ++it) {
                const double q = legendre(p + 1, z) - legendre(p - 1, z);
                const double dq = (2.0 * p + 1.0) * legendre(p, z);
                const double dz = q / dq;
                z -= dz;
                if (std::fabs(dz) < 1e-17) break;
            }
            neg[k] = z;
        }
        int c = 0;
        x[c++] = -1;
        for (int k = 0; k < h; ++k) x[c++] = neg[k];
        if (p % 2 == 0) x[c++] = 0;
        for (int k = h - 1; k >= 0; --k) x[c++] = -neg[k];
        x[c++] = 1;
    }
    w[0] = 2.0 / (p * (p + 1));
    w[p] = w[0];
    for (int i = 0; i < p / 2 + 1; ++i) {
        const double pn = legendre(p, x[i]);
        w[i] = 2.0 / (p * (p + 1) * (pn * pn));
        w[p - i] = w[i];
    }
}

// Barycentric differentiation matrix, column-major like arma
// (include/derivative_matrix.hpp:12-38 -- the same formula, kept identical
// because parity of every apply depends on it).
static std::vector<double> dmatrix(const std::vector<double>& x)
{
    const int n = (int)x.size();
    std::vector<double> bw(n, 1.0), D(n * n, 0.0);
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j)
            if (i != j) bw[i] *= x[i] - x[j];
        bw[i] = 1 / bw[i];
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            if (j != i) {
                D[i + j * n] = (bw[j] / bw[i]) / (x[i] - x[j]);
                D[i + i * n] -= D[i + j * n];
            }
    return D;
}

// ------------------------------------------------------------------ context
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct sem_ctx {
    int p = 0, N = 0, E = 0, n_nodes = 0, n_edges = 0, n_int_edges = 0, n_bnd_edges = 0,
        n_bnd_nodes = 0;
    long long n = 0, dof = 0;
    unsigned flags = 0;
    std::vector<double> x, w, D;           // D column-major
    std::vector<double> Drow_host;         // D row-major (DevMesh::Dh)
    std::vector<float> D32_host, S32_host; // FP32 D and preconditioner basis S, row-major
    std::vector<double> coords;            // [n_nodes][2]
    std::vector<int> elements;             // [E][4]
    std::vector<int> fl_host;              // DevMesh::flags, host copy
    std::vector<double> J, A, B, C;        // host metrics [E][N][N]
    DevMesh dm;
    std::vector<void*> owned;              // device allocations freed at destroy
    cudaStream_t stream = nullptr;
    int device = 0, sms = 0;
    // options
    int prec = SEM_PREC_FP64;
    double inner_tol = 1e-4;
    int guess = SEM_GUESS_ZERO;
    double timeout_ms = 2000.0;
    int max_refine = 50;
    bool profile = false;
    int precond = 0;
    int inner_fused = 1;
    double outer_scale = 1.0;
    int apply_pipeline = 1;
    int extrap_order = 1;
    int learned_step = 0;  // SEM_OPT_LEARNED_STEP
    // |r|^2 of the last learned guess's base residual: the feature scale
    // floor of the next guess (saves a read-back per stage); < 0 unknown
    double lr_nrm2 = -1.0;
    int adaptive_inner = 1;
    int resident = 1;
    // projection stage guess: basis size (0 off), slots in use, next slot,
    // Gram matrix b_i.b_j of the stored right-hand sides (proj_k^2)
    int proj_k = 0, proj_count = 0, proj_head = 0;
    std::vector<double> proj_G;
    // stage-guess history of the SDIRK drivers (persists across calls)
    long long hist_steps = 0;
    int hist_stages = 0;
    double hist_dt = 0.0;
    double hist_sig[2] = {0.0, 0.0};  // squared norms of the state the last call ended with
    // learned stage guess: network (owned by the caller) and the training
    // dataset recorded from solved stages (device workspace ds_X, ds_T)
    sem_learner* learner = nullptr;
    long long ds_cap = 0, ds_rows = 0;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    sem_stats stats{};
    // workspace
    std::unordered_map<std::string, DevBuf> ws;
    SolveOut* h_out = nullptr;  // pinned
    GridSync* h_sync = nullptr; // pinned
    double* h_lstat = nullptr;  // pinned: the last learned step's (|r|^2, theta, ratio, accepted)
    bool lr_pending = false;    // h_lstat holds a step whose statistics are not collected yet
    double* h_part = nullptr;   // pinned partials for dots
};

// accessors for the library's other translation units (sem_internal.h)
namespace semgb {
const DevMesh& ctx_mesh(const sem_ctx* c) { return c->dm; }
cudaStream_t ctx_stream(const sem_ctx* c) { return c->stream; }
void ctx_count_launches(sem_ctx* c, long long k) { c->stats.kernel_launches += k; }
int ctx_device(const sem_ctx* c) { return c->device; }
void ctx_count_fp64_apply(sem_ctx* c) { c->stats.fp64_applies++; }
int ctx_fail(int code, const char* msg) { return fail(code, msg); }
}  // namespace semgb

static int ctx_alloc(sem_ctx* c, void** p, size_t bytes)
{
    cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) return fail(SEM_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    c->owned.push_back(*p);
    return SEM_OK;
}

template <class T>
static int upload(sem_ctx* c, const std::vector<T>& v, const T** out)
{
    void* p = nullptr;
    int s = ctx_alloc(c, &p, v.size() * sizeof(T));
    if (s) return s;
    if (!v.empty()) SEM_CUDA(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    *out = (const T*)p;
    return SEM_OK;
}

// named workspace buffer of at least `bytes`, allocated on first use
static int wsbuf(sem_ctx* c, const char* name, size_t bytes, void** out)
{
    DevBuf& b = c->ws[name];
    if (b.bytes < bytes) {
        if (b.p) cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
        cudaError_t e = cudaMalloc(&b.p, std::max<size_t>(bytes, 16));
        if (e != cudaSuccess)
            return fail(SEM_ERR_CUDA, std::string("cudaMalloc(workspace): ") + cudaGetErrorString(e));
        b.bytes = bytes;
    }
    *out = b.p;
    return SEM_OK;
}

template <class T>
static int wsget(sem_ctx* c, const char* name, size_t count, T** out)
{
    void* p = nullptr;
    int s = wsbuf(c, name, count * sizeof(T), &p);
    *out = (T*)p;
    return s;
}

static bool is_device_ptr(const void* p)
{
    if (!p) return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Eigen-decomposition of a symmetric n x n matrix (row-major, overwritten):
// cyclic Jacobi rotations (Golub & Van Loan, Matrix Computations, 8.5).  On
// return A's diagonal holds the eigenvalues and V's columns the eigenvectors.
static void sym_eig_jacobi(int n, std::vector<double>& A, std::vector<double>& V)
{
    V.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int p = 0; p < n; ++p) {
            diag += A[(size_t)p * n + p] * A[(size_t)p * n + p];
            for (int q = p + 1; q < n; ++q) off += A[(size_t)p * n + q] * A[(size_t)p * n + q];
        }
        if (off <= 1e-32 * diag) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[(size_t)p * n + q];
                if (apq == 0.0) continue;
                const double theta = (A[(size_t)q * n + q] - A[(size_t)p * n + p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
                for (int k = 0; k < n; ++k) {  // columns p, q
                    const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
                    A[(size_t)k * n + p] = cs * akp - sn * akq;
                    A[(size_t)k * n + q] = sn * akp + cs * akq;
                }
                for (int k = 0; k < n; ++k) {  // rows p, q
                    const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
                    A[(size_t)p * n + k] = cs * apk - sn * aqk;
                    A[(size_t)q * n + k] = sn * apk + cs * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
                    V[(size_t)k * n + p] = cs * vkp - sn * vkq;
                    V[(size_t)k * n + q] = sn * vkp + cs * vkq;
                }
            }
    }
}

// 1-D basis of the element preconditioner: K s = lambda W s for the GLL
// stiffness K = D^T W D and mass W on [-1,1]; S(i,k) at [i*N+k] with
// S^T W S = I, S^T K S = diag(lambda).  D column-major (D(i,j) at [i+j*N]).
static void fdm_basis(int N, const std::vector<double>& w, const std::vector<double>& D, std::vector<double>& S,
                      std::vector<double>& lam)
{
    std::vector<double> B((size_t)N * N), Q;
    for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) {
            double k = 0.0;
            for (int q = 0; q < N; ++q) k += D[q + (size_t)i * N] * w[q] * D[q + (size_t)j * N];
            B[(size_t)i * N + j] = k / std::sqrt(w[i] * w[j]);
        }
    sym_eig_jacobi(N, B, Q);
    S.assign((size_t)N * N, 0.0);
    lam.assign(N, 0.0);
    for (int k = 0; k < N; ++k) {
        lam[k] = B[(size_t)k * N + k];
        for (int i = 0; i < N; ++i) S[(size_t)i * N + k] = Q[(size_t)i * N + k] / std::sqrt(w[i]);
    }
}

// Build topology (include/load_mesh.hpp:146-206) and metrics
// (include/Quad.hpp:27-55), upload everything.
static int build_ctx(sem_ctx* c, int p, int n_nodes, const double* coords, int n_el,
                     const int* elements, unsigned flags)
{
    if (p < 1 || p > MAX_N - 1) return fail(SEM_ERR_ARG, "polynomial degree must be 1..16");
    if (n_nodes <= 0 || n_el <= 0 || !coords || !elements) return fail(SEM_ERR_ARG, "empty mesh");
    if (flags & ~(SEM_FLAG_METRIC_CORRECTED | SEM_FLAG_NEUMANN)) return fail(SEM_ERR_ARG, "unknown context flag");
    const int N = p + 1, NN = N * N;
    if ((long long)n_el * NN >= (1LL << 31)) return fail(SEM_ERR_UNSUPPORTED, "mesh too large for 32-bit node indices");
    c->p = p;
    c->N = N;
    c->E = n_el;
    c->n_nodes = n_nodes;
    c->n = (long long)n_el * NN;
    c->flags = flags;
    c->coords.assign(coords, coords + 2 * (size_t)n_nodes);
    c->elements.assign(elements, elements + 4 * (size_t)n_el);
    for (int k = 0; k < 4 * n_el; ++k)
        if (elements[k] < 0 || elements[k] >= n_nodes) return fail(SEM_ERR_MESH, "corner id out of range");
    for (int e = 0; e < n_el; ++e)
        for (int a = 0; a < 4; ++a)
            for (int b = a + 1; b < 4; ++b)
                if (elements[4 * e + a] == elements[4 * e + b])
                    return fail(SEM_ERR_MESH, "element " + std::to_string(e) + " repeats a corner");
    lgl(p, c->x, c->w);
    c->D = dmatrix(c->x);

    // unique edges keyed by the sorted corner pair; first element seen owns it
    static const int emap1[] = {0, 1, 3, 0}, emap2[] = {1, 2, 2, 3};
    struct Ed { int el[2]; int side[2]; };  // side: 0..3, el[1] = -1 on the boundary; rev flag below
    std::vector<Ed> edges;
    std::vector<char> rev;
    edges.reserve(2 * (size_t)n_el + 4);
    std::unordered_map<long long, int> key2e;
    key2e.reserve(4 * (size_t)n_el);
    for (int e = 0; e < n_el; ++e)
        for (int s = 0; s < 4; ++s) {
            const int a = elements[4 * e + emap1[s]], b = elements[4 * e + emap2[s]];
            const long long key = (long long)std::min(a, b) * n_nodes + std::max(a, b);
            auto it = key2e.find(key);
            if (it == key2e.end()) {
                key2e.emplace(key, (int)edges.size());
                edges.push_back(Ed{{e, -1}, {s, -1}});
                rev.push_back(0);
            } else {
                Ed& ed = edges[it->second];
                if (ed.el[1] != -1) return fail(SEM_ERR_MESH, "an edge is shared by more than two elements");
                const int n1 = elements[4 * ed.el[0] + emap1[ed.side[0]]];
                ed.el[1] = e;
                ed.side[1] = s;
                rev[it->second] = (a == n1) ? 0 : 1;  // load_mesh.hpp:164-171
            }
        }
    c->n_edges = (int)edges.size();
    // Neumann context: boundary sides are owned and partnerless, boundary
    // corners ordinary (node_bnd stays clear); on_bnd marks them for the count
    const bool neumann = (flags & SEM_FLAG_NEUMANN) != 0;
    std::vector<int> fl(n_el, 0), sbase(4 * (size_t)n_el, -1), sstep(4 * (size_t)n_el, 0);
    std::vector<char> node_bnd(n_nodes, 0), on_bnd(n_nodes, 0);
    auto side_pos = [&](int e, int s, int k) -> long long {  // flat index of node k on side s
        const long long b = (long long)e * NN;
        switch (s) {
            case 0: return b + k;
            case 1: return b + (N - 1) + (long long)k * N;
            case 2: return b + k + (long long)(N - 1) * N;
            default: return b + (long long)k * N;
        }
    };
    for (size_t q = 0; q < edges.size(); ++q) {
        const Ed& ed = edges[q];
        if (ed.el[1] < 0) {
            ++c->n_bnd_edges;
            on_bnd[elements[4 * ed.el[0] + emap1[ed.side[0]]]] = 1;
            on_bnd[elements[4 * ed.el[0] + emap2[ed.side[0]]]] = 1;
            if (neumann) {
                fl[ed.el[0]] |= (1 << ed.side[0]) | (65536 << ed.side[0]);
                continue;
            }
            fl[ed.el[0]] |= (1 << ed.side[0]) | (16 << ed.side[0]);
            node_bnd[elements[4 * ed.el[0] + emap1[ed.side[0]]]] = 1;
            node_bnd[elements[4 * ed.el[0] + emap2[ed.side[0]]]] = 1;
            continue;
        }
        ++c->n_int_edges;
        fl[ed.el[0]] |= (1 << ed.side[0]);
        for (int h = 0; h < 2; ++h) {
            const int e = ed.el[h], s = ed.side[h];
            const int eo = ed.el[1 - h], so = ed.side[1 - h];
            // node k of (e,s) pairs with node k (same orientation) or N-1-k of (eo,so)
            if (!rev[q]) {
                sbase[4 * e + s] = (int)side_pos(eo, so, 0);
                sstep[4 * e + s] = (int)(side_pos(eo, so, 1) - side_pos(eo, so, 0));
            } else {
                sbase[4 * e + s] = (int)side_pos(eo, so, N - 1);
                sstep[4 * e + s] = -(int)(side_pos(eo, so, 1) - side_pos(eo, so, 0));
            }
        }
    }
    // corner copies in element order (load_mesh.hpp:123-143)
    static const int cmi[] = {0, 1, 1, 0}, cmj[] = {0, 0, 1, 1};
    std::vector<int> nptr(n_nodes + 1, 0), nflat(4 * (size_t)n_el), cnode(4 * (size_t)n_el),
        csrc(4 * (size_t)n_el);
    for (int k = 0; k < 4 * n_el; ++k) nptr[elements[k] + 1]++;
    for (int k = 0; k < n_nodes; ++k) nptr[k + 1] += nptr[k];
    std::vector<int> fill(n_nodes, 0);
    for (int e = 0; e < n_el; ++e)
        for (int cc = 0; cc < 4; ++cc) {
            const int node = elements[4 * e + cc];
            const int flat = e * NN + cmi[cc] * (N - 1) + cmj[cc] * (N - 1) * N;
            nflat[nptr[node] + fill[node]++] = flat;
            cnode[4 * e + cc] = node;
        }
    for (int e = 0; e < n_el; ++e)
        for (int cc = 0; cc < 4; ++cc) {
            const int node = cnode[4 * e + cc];
            const int flat = e * NN + cmi[cc] * (N - 1) + cmj[cc] * (N - 1) * N;
            csrc[4 * e + cc] = nflat[nptr[node]];
            if (nflat[nptr[node]] == flat) fl[e] |= (256 << cc);
            if (node_bnd[node]) fl[e] |= (4096 << cc);
        }
    for (int k = 0; k < n_nodes; ++k) c->n_bnd_nodes += on_bnd[k];
    // corner copies in CSR order per element corner (the gathers read them
    // with one dependent load instead of three)
    std::vector<int> corner_nb((size_t)n_el * 4 * CORNER_NB_MAX, -1), corner_cnt4(n_el, 0);
    std::vector<int> node_nb((size_t)n_nodes * CORNER_NB_MAX, -1);
    for (int node = 0; node < n_nodes; ++node) {
        const int q0 = nptr[node], cnt = nptr[node + 1] - q0;
        int* dst = &node_nb[(size_t)node * CORNER_NB_MAX];
        if (cnt > CORNER_NB_MAX)
            dst[0] = -2;
        else
            for (int q = 0; q < cnt; ++q) dst[q] = nflat[q0 + q];
    }
    for (int e = 0; e < n_el; ++e)
        for (int cc = 0; cc < 4; ++cc) {
            const int node = cnode[4 * e + cc];
            const int q0 = nptr[node], cnt = nptr[node + 1] - q0;
            if (cnt > 255) return fail(SEM_ERR_MESH, "a corner node is shared by more than 255 elements");
            corner_cnt4[e] |= cnt << (8 * cc);
            int* dst = &corner_nb[((size_t)e * 4 + cc) * CORNER_NB_MAX];
            if (cnt > CORNER_NB_MAX)
                dst[0] = -2;
            else
                for (int q = 0; q < cnt; ++q) dst[q] = nflat[q0 + q];
        }
    // ring tables of the in-place assembly and the pipelined apply's gather
    const int R = 4 * (N - 1);
    std::vector<int> ring_src((size_t)n_el * R, -1), bnd_flat;
    std::vector<int2> edge_pairs;
    for (int e = 0; e < n_el; ++e) {
        for (int r = 0; r < R; ++r) {
            int ii, jj;
            if (r < N - 1) {
                ii = r;
                jj = 0;
            } else if (r < 2 * (N - 1)) {
                ii = N - 1;
                jj = r - (N - 1);
            } else if (r < 3 * (N - 1)) {
                ii = N - 1 - (r - 2 * (N - 1));
                jj = N - 1;
            } else {
                ii = 0;
                jj = N - 1 - (r - 3 * (N - 1));
            }
            const bool ib = (ii == 0 || ii == N - 1), jb = (jj == 0 || jj == N - 1);
            int src = -1;
            if (ib && jb) {
                const int cc = (jj == 0) ? (ii == 0 ? 0 : 1) : (ii == 0 ? 3 : 2);
                if (!(fl[e] & (256 << cc)) && !(fl[e] & (4096 << cc))) src = csrc[4 * e + cc];
            } else {
                const int sd = jb ? (jj == 0 ? 0 : 2) : (ii == N - 1 ? 1 : 3);
                const int k = jb ? ii : jj;
                if (!(fl[e] & (1 << sd)) && !(fl[e] & (16 << sd)))
                    src = (int)(sbase[4 * e + sd] + (long long)k * sstep[4 * e + sd]);
            }
            ring_src[(size_t)e * R + r] = src;
        }
        for (int sd = 0; sd < 4; ++sd) {
            const bool bnd = fl[e] & (16 << sd), own = fl[e] & (1 << sd), lone = fl[e] & (65536 << sd);
            for (int k = 1; k < N - 1; ++k) {
                if (bnd)
                    bnd_flat.push_back((int)side_pos(e, sd, k));
                else if (own && !lone)
                    edge_pairs.push_back(
                        make_int2((int)side_pos(e, sd, k), (int)(sbase[4 * e + sd] + (long long)k * sstep[4 * e + sd])));
            }
        }
    }
    c->dof = (long long)n_nodes + (long long)c->n_edges * (N - 2) + (long long)n_el * (N - 2) * (N - 2);
    // side pairs inside one batch of the pipelined FP32 apply go last in
    // edge_pairs and into per-batch tables of batch-local offsets
    const int bK = bulk_k<float, OP_RES>(N);
    const long long bN = (long long)bK * NN;
    const long long nbatch = (n_el + bK - 1) / bK;
    std::vector<int> bulk_pair_ptr(nbatch + 1, 0), bulk_pairs;
    long long n_pairs_x = 0;
    {
        auto internal = [&](const int2& pr) { return (long long)pr.x / bN == (long long)pr.y / bN; };
        std::stable_partition(edge_pairs.begin(), edge_pairs.end(), [&](const int2& pr) { return !internal(pr); });
        for (const int2& pr : edge_pairs) {
            if (!internal(pr)) {
                ++n_pairs_x;
                continue;
            }
            bulk_pair_ptr[pr.x / bN + 1]++;
        }
        for (long long b = 0; b < nbatch; ++b) bulk_pair_ptr[b + 1] += bulk_pair_ptr[b];
        bulk_pairs.assign(bulk_pair_ptr[nbatch], 0);
        std::vector<int> fill(nbatch, 0);
        for (long long q = n_pairs_x; q < (long long)edge_pairs.size(); ++q) {
            const int2 pr = edge_pairs[q];
            const long long b = pr.x / bN;
            const int o = (int)(pr.x - b * bN), x = (int)(pr.y - b * bN);
            bulk_pairs[bulk_pair_ptr[b] + fill[b]++] = (o << 16) | x;
        }
    }

    // metrics, include/Quad.hpp:39-54 (C as the reference writes it unless corrected)
    const bool corrected = (flags & SEM_FLAG_METRIC_CORRECTED) != 0;
    c->J.assign(c->n, 0.0);
    c->A.assign(c->n, 0.0);
    c->B.assign(c->n, 0.0);
    c->C.assign(c->n, 0.0);
    std::vector<double> g11(c->n), g12(c->n), g22(c->n), ms(c->n);
    std::vector<float> geo((size_t)n_el * 8);  // corner differences of the on-the-fly FP32 apply
    const std::vector<double>& z = c->x;
    for (int e = 0; e < n_el; ++e) {
        double xs[4], ys[4];
        for (int k = 0; k < 4; ++k) {
            xs[k] = coords[2 * elements[4 * e + k]];
            ys[k] = coords[2 * elements[4 * e + k] + 1];
        }
        const double gd[8] = {xs[1] - xs[0], xs[2] - xs[3], xs[3] - xs[0], xs[2] - xs[1],
                              ys[1] - ys[0], ys[2] - ys[3], ys[3] - ys[0], ys[2] - ys[1]};
        for (int k = 0; k < 8; ++k) geo[(size_t)e * 8 + k] = (float)gd[k];
        double Xxi[MAX_N], Yxi[MAX_N], Xeta[MAX_N], Yeta[MAX_N];
        for (int i = 0; i < N; ++i) {
            Xxi[i] = 0.25 * ((1 - z[i]) * (xs[1] - xs[0]) + (1 + z[i]) * (xs[2] - xs[3]));
            Yxi[i] = 0.25 * ((1 - z[i]) * (ys[1] - ys[0]) + (1 + z[i]) * (ys[2] - ys[3]));
            Xeta[i] = 0.25 * ((1 - z[i]) * (xs[3] - xs[0]) + (1 + z[i]) * (xs[2] - xs[1]));
            Yeta[i] = 0.25 * ((1 - z[i]) * (ys[3] - ys[0]) + (1 + z[i]) * (ys[2] - ys[1]));
        }
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                const size_t k = (size_t)e * NN + i + (size_t)j * N;
                const double Jv = Xxi[j] * Yeta[i] - Xeta[i] * Yxi[j];
                const double Av = (Yeta[i] * Yeta[i] + Xeta[i] * Xeta[i]) / Jv;
                const double Bv = (Yeta[i] * Yxi[j] + Xeta[i] * Xxi[j]) / Jv;
                const double yx = corrected ? Yxi[j] : Yxi[i];
                const double Cv = (yx * yx + Xxi[j] * Xxi[j]) / Jv;
                c->J[k] = Jv;
                c->A[k] = Av;
                c->B[k] = Bv;
                c->C[k] = Cv;
                const double ww = c->w[i] * c->w[j];
                g11[k] = ww * Av;
                g12[k] = ww * Bv;
                g22[k] = ww * Cv;
                ms[k] = ww * Jv;
            }
    }
    // diagonals of the assembled stiffness and lumped mass (continuous format),
    // for the diagonal preconditioner.  Element-local diagonal of the weak
    // Laplacian: sum_k D(k,i)^2 g11(k,j) + sum_k D(k,j)^2 g22(i,k) - 2 D(i,i) D(j,j) g12(i,j)
    std::vector<double> kloc(c->n), kdiag(c->n), mdiag(c->n);
    for (int e = 0; e < n_el; ++e)
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                const size_t b = (size_t)e * NN;
                double s = 0.0;
                for (int k = 0; k < N; ++k) {
                    const double dki = c->D[k + i * N], dkj = c->D[k + j * N];
                    s += dki * dki * g11[b + k + (size_t)j * N] + dkj * dkj * g22[b + i + (size_t)k * N];
                }
                s -= 2.0 * c->D[i + i * N] * c->D[j + j * N] * g12[b + i + (size_t)j * N];
                kloc[b + i + (size_t)j * N] = s;
            }
    auto assemble = [&](const std::vector<double>& loc, std::vector<double>& out) {
        for (int e = 0; e < n_el; ++e)
            for (int j = 0; j < N; ++j)
                for (int i = 0; i < N; ++i) {
                    const size_t f = (size_t)e * NN + i + (size_t)j * N;
                    const bool ib = (i == 0 || i == N - 1), jb = (j == 0 || j == N - 1);
                    double v = loc[f];
                    if (ib && jb) {
                        const int cc = (j == 0) ? (i == 0 ? 0 : 1) : (i == 0 ? 3 : 2);
                        const int node = cnode[4 * e + cc];
                        v = 0.0;
                        for (int q = nptr[node]; q < nptr[node + 1]; ++q) v += loc[nflat[q]];
                    } else if (ib || jb) {
                        const int sd = jb ? (j == 0 ? 0 : 2) : (i == N - 1 ? 1 : 3);
                        const int k = jb ? i : j;
                        if (!(fl[e] & ((16 | 65536) << sd)))
                            v += loc[(size_t)(sbase[4 * e + sd] + (long long)k * sstep[4 * e + sd])];
                    }
                    out[f] = v;
                }
    };
    assemble(kloc, kdiag);
    assemble(ms, mdiag);
    // element preconditioner data: 1-D basis and each element's rectangle
    // approximation (half widths from the mean lengths of opposite sides)
    std::vector<double> fS, fL;
    fdm_basis(N, c->w, c->D, fS, fL);
    std::vector<float4> fel(n_el);
    for (int e = 0; e < n_el; ++e) {
        double cx[4], cy[4];
        for (int k = 0; k < 4; ++k) {
            cx[k] = coords[2 * (size_t)elements[4 * (size_t)e + k]];
            cy[k] = coords[2 * (size_t)elements[4 * (size_t)e + k] + 1];
        }
        auto len = [&](int a, int b) { return std::hypot(cx[b] - cx[a], cy[b] - cy[a]); };
        const double ax = 0.25 * (len(0, 1) + len(3, 2)), ay = 0.25 * (len(0, 3) + len(1, 2));
        fel[e] = make_float4((float)(ax * ay), (float)(ay / ax), (float)(ax / ay), 0.f);
    }

    c->fl_host = fl;
    // device copies
    DevMesh& d = c->dm;
    d.N = N;
    d.E = n_el;
    d.n_nodes = n_nodes;
    d.n = c->n;
    std::vector<double> Drow(NN);
    std::vector<float> Drowf(NN);
    for (int i = 0; i < N; ++i)
        for (int k = 0; k < N; ++k) {
            Drow[i * N + k] = c->D[i + k * N];
            Drowf[i * N + k] = (float)c->D[i + k * N];
        }
    c->Drow_host = Drow;
    d.Dh = c->Drow_host.data();
    d.zh = c->x.data();
    d.wh = c->w.data();
    d.corrected = corrected ? 1 : 0;
    auto tof = [](const std::vector<double>& v) {
        std::vector<float> f(v.size());
        for (size_t i = 0; i < v.size(); ++i) f[i] = (float)v[i];
        return f;
    };
    c->D32_host = Drowf;
    c->S32_host = tof(fS);
    int s = 0;
    if ((s = upload(c, fl, &d.flags)) || (s = upload(c, sbase, &d.side_base)) ||
        (s = upload(c, sstep, &d.side_step)) || (s = upload(c, csrc, &d.corner_src)) ||
        (s = upload(c, cnode, &d.corner_node)) || (s = upload(c, nptr, &d.node_ptr)) ||
        (s = upload(c, nflat, &d.node_flat)) || (s = upload(c, Drow, &d.D64)) ||
        (s = upload(c, Drowf, &d.D32)) || (s = upload(c, g11, &d.g11)) || (s = upload(c, g12, &d.g12)) ||
        (s = upload(c, g22, &d.g22)) || (s = upload(c, ms, &d.mass)) ||
        (s = upload(c, tof(g11), &d.g11f)) || (s = upload(c, tof(g12), &d.g12f)) ||
        (s = upload(c, tof(g22), &d.g22f)) || (s = upload(c, tof(ms), &d.massf)) ||
        (s = upload(c, kdiag, &d.kdiag)) || (s = upload(c, mdiag, &d.mdiag)) ||
        (s = upload(c, fS, &d.fdmS64)) || (s = upload(c, tof(fS), &d.fdmS32)) ||
        (s = upload(c, fL, &d.fdmL64)) || (s = upload(c, tof(fL), &d.fdmL32)) || (s = upload(c, fel, &d.fdm_el)) ||
        (s = upload(c, ring_src, &d.ring_src)) || (s = upload(c, edge_pairs, &d.edge_pairs)) ||
        (s = upload(c, corner_nb, &d.corner_nb)) || (s = upload(c, corner_cnt4, &d.corner_cnt4)) ||
        (s = upload(c, node_nb, &d.node_nb)) ||
        (s = upload(c, bulk_pair_ptr, &d.bulk_pair_ptr)) ||
        (!bulk_pairs.empty() && (s = upload(c, bulk_pairs, &d.bulk_pairs))) ||
        (s = upload(c, bnd_flat, &d.bnd_flat)) || (s = upload(c, node_bnd, &d.node_bnd)) ||
        (s = upload(c, geo, &d.geo32)))
        return s;
    d.n_pairs = (long long)edge_pairs.size();
    d.n_pairs_x = n_pairs_x;
    d.bulk_K = bK;
    d.n_bnd = (long long)bnd_flat.size();
    {
        void* p = nullptr;
        if ((s = ctx_alloc(c, &p, sizeof(int)))) return s;
        SEM_CUDA(cudaMemset(p, 0, sizeof(int)));
        d.dev_err = (int*)p;
    }
    SEM_CUDA(cudaMallocHost((void**)&c->h_out, sizeof(SolveOut)));
    SEM_CUDA(cudaMallocHost((void**)&c->h_sync, sizeof(GridSync)));
    SEM_CUDA(cudaMallocHost((void**)&c->h_part, sizeof(double) * 152 * 64));
    SEM_CUDA(cudaMallocHost((void**)&c->h_lstat, sizeof(double) * 4));
    return SEM_OK;
}

// ------------------------------------------------------------ C ABI: misc
extern "C" int sem_version(void) { return SEM_GB300_VERSION; }

extern "C" const char* sem_status_string(int s)
{
    switch (s) {
        case SEM_OK: return "ok";
        case SEM_ERR_ARG: return "invalid argument";
        case SEM_ERR_CUDA: return "CUDA error";
        case SEM_ERR_MESH: return "invalid mesh";
        case SEM_ERR_IO: return "mesh folder unreadable";
        case SEM_ERR_DEVICE_WAIT: return "device-side wait timed out";
        case SEM_ERR_UNSUPPORTED: return "unsupported";
        case SEM_ERR_NO_DEVICE: return "no CUDA device";
        default: return "unknown status";
    }
}

extern "C" const char* sem_last_error(void) { return g_last_error.c_str(); }

// ------------------------------------------------------------ C ABI: mesh
extern "C" int sem_ctx_create(sem_ctx** out, int p, int n_nodes, const double* coords, int n_el,
                              const int* elements, unsigned flags)
{
    if (!out) return fail(SEM_ERR_ARG, "ctx pointer is null");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(SEM_ERR_NO_DEVICE, "no CUDA device visible");
    }
    sem_ctx* c = new sem_ctx();
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device);
    int s = build_ctx(c, p, n_nodes, coords, n_el, elements, flags);
    if (s) {
        sem_ctx_destroy(c);
        return s;
    }
    *out = c;
    return SEM_OK;
}

extern "C" int sem_ctx_load(sem_ctx** out, int p, const char* folder, unsigned flags)
{
    if (!folder) return fail(SEM_ERR_ARG, "folder is null");
    std::string f(folder);
    std::ifstream info(f + "/info.txt");
    if (!info.is_open()) return fail(SEM_ERR_IO, "could not open info file.");  // load_mesh.hpp:92-93
    int n_nodes = 0, n_el = 0;
    info >> n_nodes >> n_el;
    if (n_nodes <= 0 || n_el <= 0) return fail(SEM_ERR_IO, "bad info.txt");
    std::ifstream co(f + "/coordinates.txt");
    if (!co.is_open()) return fail(SEM_ERR_IO, "could not open coordinate file.");
    std::vector<double> coords(2 * (size_t)n_nodes);
    for (auto& v : coords)
        if (!(co >> v)) return fail(SEM_ERR_IO, "coordinates.txt too short");
    std::ifstream el(f + "/elements.txt");
    if (!el.is_open()) return fail(SEM_ERR_IO, "could not open element file.");
    std::vector<int> elements(4 * (size_t)n_el);
    for (auto& v : elements)
        if (!(el >> v)) return fail(SEM_ERR_IO, "elements.txt too short");
    return sem_ctx_create(out, p, n_nodes, coords.data(), n_el, elements.data(), flags);
}

extern "C" int sem_ctx_destroy(sem_ctx* c)
{
    if (!c) return SEM_OK;
    if (c->stream) cudaStreamSynchronize(c->stream);
    else cudaDeviceSynchronize();
    for (void* p : c->owned) cudaFree(p);
    for (auto& kv : c->ws)
        if (kv.second.p) cudaFree(kv.second.p);
    if (c->h_out) cudaFreeHost(c->h_out);
    if (c->h_sync) cudaFreeHost(c->h_sync);
    if (c->h_lstat) cudaFreeHost(c->h_lstat);
    if (c->h_part) cudaFreeHost(c->h_part);
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    delete c;
    return SEM_OK;
}

extern "C" int sem_ctx_get_info(const sem_ctx* c, sem_mesh_info* info)
{
    if (!c || !info) return fail(SEM_ERR_ARG, "null argument");
    info->p = c->p;
    info->N = c->N;
    info->n_elements = c->E;
    info->n_nodes = c->n_nodes;
    info->n_edges = c->n_edges;
    info->n_interior_edges = c->n_int_edges;
    info->n_boundary_edges = c->n_bnd_edges;
    info->n_boundary_nodes = c->n_bnd_nodes;
    info->n_local = c->n;
    info->dof = c->dof;
    return SEM_OK;
}

extern "C" int sem_ctx_set_stream(sem_ctx* c, void* st)
{
    if (!c) return fail(SEM_ERR_ARG, "null ctx");
    c->stream = (cudaStream_t)st;
    return SEM_OK;
}

extern "C" int sem_ctx_set_option(sem_ctx* c, int opt, double v)
{
    if (!c) return fail(SEM_ERR_ARG, "null ctx");
    switch (opt) {
        case SEM_OPT_SOLVE_PRECISION:
            if (v != SEM_PREC_FP64 && v != SEM_PREC_MIXED) return fail(SEM_ERR_ARG, "bad precision");
            c->prec = (int)v;
            return SEM_OK;
        case SEM_OPT_INNER_TOL:
            if (!(v > 0 && v < 1)) return fail(SEM_ERR_ARG, "inner tolerance must be in (0,1)");
            c->inner_tol = v;
            return SEM_OK;
        case SEM_OPT_STAGE_GUESS:
            if (v != SEM_GUESS_ZERO && v != SEM_GUESS_EXTRAPOLATE && v != SEM_GUESS_LEARNED)
                return fail(SEM_ERR_ARG, "bad guess mode");
            c->guess = (int)v;
            c->hist_steps = 0;  // a new guess mode starts a new history
            c->proj_count = c->proj_head = 0;
            return SEM_OK;
        case SEM_OPT_WAIT_TIMEOUT_MS:
            if (!(v > 0)) return fail(SEM_ERR_ARG, "timeout must be positive");
            c->timeout_ms = v;
            return SEM_OK;
        case SEM_OPT_MAX_REFINE:
            if (!(v >= 1)) return fail(SEM_ERR_ARG, "max refine must be >= 1");
            c->max_refine = (int)v;
            return SEM_OK;
        case SEM_OPT_REFINE_TOL_SCALE:
            if (!(v > 0 && v <= 1)) return fail(SEM_ERR_ARG, "refinement tolerance scale must be in (0,1]");
            c->outer_scale = v;
            return SEM_OK;
        case SEM_OPT_ADAPTIVE_INNER:
            if (v != 0 && v != 1) return fail(SEM_ERR_ARG, "adaptive inner tolerance must be 0 or 1");
            c->adaptive_inner = (int)v;
            return SEM_OK;
        case SEM_OPT_EXTRAP_ORDER:
            if (v != 1 && v != 2) return fail(SEM_ERR_ARG, "extrapolation order must be 1 or 2");
            c->extrap_order = (int)v;
            return SEM_OK;
        case SEM_OPT_APPLY_PIPELINE:
            if (v != 0 && v != 1 && v != 2) return fail(SEM_ERR_ARG, "apply pipeline must be 0, 1 or 2");
            c->apply_pipeline = (int)v;
            return SEM_OK;
        case SEM_OPT_LEARNED_STEP:
            if (v != 0 && v != 1) return fail(SEM_ERR_ARG, "learned step must be 0 or 1");
            c->learned_step = (int)v;
            return SEM_OK;
        case SEM_OPT_PROJECT:
            if (!(v >= 0 && v <= PROJ_MAX) || v != (double)(int)v)
                return fail(SEM_ERR_ARG, "projection basis size must be an integer in [0, 24]");
            c->proj_k = (int)v;
            c->proj_count = c->proj_head = 0;
            c->proj_G.assign((size_t)c->proj_k * c->proj_k, 0.0);
            return SEM_OK;
        case SEM_OPT_RESIDENT:
            if (v != 0 && v != 1) return fail(SEM_ERR_ARG, "resident inner solve must be 0 or 1");
            c->resident = (int)v;
            return SEM_OK;
        case SEM_OPT_INNER_ITERATION:
            if (v != 0 && v != 1) return fail(SEM_ERR_ARG, "inner iteration must be 0 or 1");
            c->inner_fused = (int)v;
            return SEM_OK;
        case SEM_OPT_PRECOND:
            if (v != SEM_PRECOND_NONE && v != SEM_PRECOND_DIAG && v != SEM_PRECOND_FDM)
                return fail(SEM_ERR_ARG, "bad preconditioner");
            c->precond = (int)v;
            return SEM_OK;
        case SEM_OPT_PROFILE:
            c->profile = v != 0;
            if (c->profile && !c->ev[0]) {
                SEM_CUDA(cudaEventCreate(&c->ev[0]));
                SEM_CUDA(cudaEventCreate(&c->ev[1]));
            }
            return SEM_OK;
        default: return fail(SEM_ERR_ARG, "unknown option");
    }
}

extern "C" int sem_ctx_get_stats(const sem_ctx* c, sem_stats* s)
{
    if (!c || !s) return fail(SEM_ERR_ARG, "null argument");
    *s = c->stats;
    return SEM_OK;
}

extern "C" int sem_ctx_get_quadrature(const sem_ctx* c, double* x, double* w, double* D)
{
    if (!c) return fail(SEM_ERR_ARG, "null ctx");
    if (x) std::memcpy(x, c->x.data(), sizeof(double) * c->N);
    if (w) std::memcpy(w, c->w.data(), sizeof(double) * c->N);
    if (D) std::memcpy(D, c->D.data(), sizeof(double) * c->N * c->N);
    return SEM_OK;
}

extern "C" int sem_ctx_get_metrics(const sem_ctx* c, double* J, double* A, double* B, double* C)
{
    if (!c) return fail(SEM_ERR_ARG, "null ctx");
    const size_t b = sizeof(double) * c->n;
    if (J) std::memcpy(J, c->J.data(), b);
    if (A) std::memcpy(A, c->A.data(), b);
    if (B) std::memcpy(B, c->B.data(), b);
    if (C) std::memcpy(C, c->C.data(), b);
    return SEM_OK;
}

extern "C" int sem_ctx_get_node_coords(const sem_ctx* c, double* X, double* Y)
{
    if (!c || !X || !Y) return fail(SEM_ERR_ARG, "null argument");
    const int N = c->N;
    for (int e = 0; e < c->E; ++e) {
        double xs[4], ys[4];
        for (int k = 0; k < 4; ++k) {
            xs[k] = c->coords[2 * c->elements[4 * e + k]];
            ys[k] = c->coords[2 * c->elements[4 * e + k] + 1];
        }
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                const double xi = c->x[i], eta = c->x[j];
                const size_t k = (size_t)e * N * N + i + (size_t)j * N;
                X[k] = 0.25 * (xs[0] * (1 - xi) * (1 - eta) + xs[1] * (1 + xi) * (1 - eta) +
                               xs[2] * (1 + xi) * (1 + eta) + xs[3] * (1 - xi) * (1 + eta));
                Y[k] = 0.25 * (ys[0] * (1 - xi) * (1 - eta) + ys[1] * (1 + xi) * (1 - eta) +
                               ys[2] * (1 + xi) * (1 + eta) + ys[3] * (1 - xi) * (1 + eta));
            }
    }
    return SEM_OK;
}

// --------------------------------------------------- C ABI: gather-scatter
#define SEM_CHECK_CTX(c) \
    if (!(c)) return fail(SEM_ERR_ARG, "null ctx")
#define SEM_LAUNCH(expr)                                                                       \
    do {                                                                                       \
        c->stats.kernel_launches++;                                                            \
        cudaError_t e_ = (expr);                                                               \
        if (e_ != cudaSuccess) return fail(SEM_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e_)); \
    } while (0)

extern "C" int sem_unmask(sem_ctx* c, double* a)
{
    SEM_CHECK_CTX(c);
    if (!a) return fail(SEM_ERR_ARG, "null field");
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) { return launch_unmask<decltype(nv)::value>(c->dm, false, a, c->stream); }));
    return SEM_OK;
}

extern "C" int sem_mask(sem_ctx* c, double* a)
{
    SEM_CHECK_CTX(c);
    if (!a) return fail(SEM_ERR_ARG, "null field");
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) { return launch_mask<decltype(nv)::value>(c->dm, false, a, c->stream); }));
    return SEM_OK;
}

extern "C" int sem_global_sum(sem_ctx* c, double* a)
{
    SEM_CHECK_CTX(c);
    if (!a) return fail(SEM_ERR_ARG, "null field");
    double* tmp = nullptr;
    int s = wsget(c, "gs_tmp", c->n, &tmp);
    if (s) return s;
    SEM_CUDA(cudaMemcpyAsync(tmp, a, sizeof(double) * c->n, cudaMemcpyDeviceToDevice, c->stream));
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
        return launch_dss<decltype(nv)::value>(c->dm, false, DSS_SUM, 1.0, tmp, a, c->stream);
    }));
    return SEM_OK;
}

static bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// the flag a pipelined apply sets when one of its bounded waits expired;
// reported (and cleared) at the next synchronising call
static int check_dev_err(sem_ctx* c)
{
    int h = 0;
    SEM_CUDA(cudaMemcpyAsync(&h, c->dm.dev_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    SEM_CUDA(cudaStreamSynchronize(c->stream));
    if (h) {
        SEM_CUDA(cudaMemsetAsync(c->dm.dev_err, 0, sizeof(int), c->stream));
        return fail(SEM_ERR_DEVICE_WAIT, "a bulk-copy wait of an operator apply timed out");
    }
    return SEM_OK;
}

static long long timeout_ns(const sem_ctx* c) { return (long long)(c->timeout_ms * 1e6); }

static int dot_dev(sem_ctx* c, const double* a, const double* b, double* result)
{
    double* part = nullptr;
    int s = wsget(c, "dot_part", 152 * 64, &part);
    if (s) return s;
    int used = 0;
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
        return launch_dot<decltype(nv)::value>(c->dm, a, b, part, 152 * 64, &used, c->stream);
    }));
    SEM_CUDA(cudaMemcpyAsync(c->h_part, part, sizeof(double) * used, cudaMemcpyDeviceToHost, c->stream));
    SEM_CUDA(cudaStreamSynchronize(c->stream));
    double acc = 0.0;
    for (int i = 0; i < used; ++i) acc += c->h_part[i];
    *result = acc;
    return SEM_OK;
}

extern "C" int sem_dot(sem_ctx* c, const double* a, const double* b, double* result)
{
    SEM_CHECK_CTX(c);
    if (!a || !b || !result) return fail(SEM_ERR_ARG, "null argument");
    const int s = dot_dev(c, a, b, result);
    return s ? s : check_dev_err(c);
}

extern "C" int sem_vec_axpby(sem_ctx* c, long long n, double a, const double* x, double b,
                             const double* y, double* out)
{
    SEM_CHECK_CTX(c);
    if (n < 0 || (n > 0 && (!x || !out))) return fail(SEM_ERR_ARG, "bad vector arguments");
    if (n == 0) return SEM_OK;
    k_axpby<<<grid_1d(n), 256, 0, c->stream>>>(n, a, x, b, y, out);
    c->stats.kernel_launches++;
    SEM_CUDA(cudaGetLastError());
    return SEM_OK;
}

// --------------------------------------------------------- C ABI: operators
// element-local op (input gathered with unmask semantics), then DSS + mask
static bool overlap(const void* a, const void* b, size_t bytes)
{
    if (!a || !b) return false;
    const char *x = (const char*)a, *y = (const char*)b;
    return x < y + bytes && y < x + bytes;
}

// the apply may write its element-local result straight into the outputs and
// assemble them in place when no output overlaps an input (the element
// kernel gathers inputs across elements)
static bool apply_direct(const sem_ctx* c, size_t word, const void* pot, const void* in0, const void* in1,
                         const void* out0, const void* out1)
{
    const size_t b = word * (size_t)c->n;
    const void* ins[3] = {pot, in0, in1};
    const void* outs[2] = {out0, out1};
    for (const void* o : outs)
        for (const void* i : ins)
            if (overlap(o, i, b)) return false;
    return !overlap(out0, out1, b);
}

static int apply_galerkin(sem_ctx* c, int op, const double* pot, double alpha, const double* in0,
                          const double* in1, double* out0, double* out1, double scale = 1.0)
{
    const int nc = (op == OP_RES || op == OP_F) ? 2 : 1;
    if (scale == 1.0 && apply_direct(c, sizeof(double), pot, in0, in1, out0, nc == 2 ? out1 : nullptr)) {
        // FP64: the one-pass kernel (FP64-pipe bound, not memory bound)
        SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
            return launch_apply<decltype(nv)::value>(c->dm, op, false, pot, alpha, in0, in1, out0, out1, true,
                                                     c->stream);
        }));
        SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
            return launch_ring<decltype(nv)::value>(c->dm, false, DSS_MASK, out0, nc == 2 ? out1 : nullptr, false,
                                                    c->stream);
        }));
        c->stats.fp64_applies++;
        return SEM_OK;
    }
    double* Y = nullptr;
    int s = wsget(c, "apply_Y", 2 * c->n, &Y);
    if (s) return s;
    double* Y1 = Y + c->n;
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
        return launch_apply<decltype(nv)::value>(c->dm, op, false, pot, alpha, in0, in1, Y, Y1, true, c->stream);
    }));
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
        return launch_dss<decltype(nv)::value>(c->dm, false, DSS_MASK, scale, Y, out0, c->stream);
    }));
    if (nc == 2)
        SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
            return launch_dss<decltype(nv)::value>(c->dm, false, DSS_MASK, scale, Y1, out1, c->stream);
        }));
    c->stats.fp64_applies++;
    return SEM_OK;
}

extern "C" int sem_gproj(sem_ctx* c, const double* u, double* out)
{
    SEM_CHECK_CTX(c);
    if (!u || !out) return fail(SEM_ERR_ARG, "null field");
    return apply_galerkin(c, OP_MASS, nullptr, 0.0, u, nullptr, out, nullptr);
}

extern "C" int sem_apply_laplace(sem_ctx* c, const double* u, double* out)
{
    SEM_CHECK_CTX(c);
    if (!u || !out) return fail(SEM_ERR_ARG, "null field");
    return apply_galerkin(c, OP_LAPLACE, nullptr, 0.0, u, nullptr, out, nullptr);
}

extern "C" int sem_apply_helmholtz(sem_ctx* c, const double* cf, const double* u, double* out)
{
    SEM_CHECK_CTX(c);
    if (!cf || !u || !out) return fail(SEM_ERR_ARG, "null field");
    return apply_galerkin(c, OP_HELM, cf, 0.0, u, nullptr, out, nullptr);
}

extern "C" int sem_apply_schro_res(sem_ctx* c, const double* V, double alpha, const double* qr,
                                   const double* qi, double* yr, double* yi)
{
    SEM_CHECK_CTX(c);
    if (!V || !qr || !qi || !yr || !yi) return fail(SEM_ERR_ARG, "null field");
    return apply_galerkin(c, OP_RES, V, alpha, qr, qi, yr, yi);
}

extern "C" int sem_apply_schro_f(sem_ctx* c, const double* V, const double* qr, const double* qi,
                                 double* yr, double* yi)
{
    SEM_CHECK_CTX(c);
    if (!V || !qr || !qi || !yr || !yi) return fail(SEM_ERR_ARG, "null field");
    return apply_galerkin(c, OP_F, V, 0.0, qr, qi, yr, yi);
}

extern "C" int sem_apply_schro_res_f32(sem_ctx* c, const float* V, float alpha, const float* qr,
                                       const float* qi, float* yr, float* yi)
{
    SEM_CHECK_CTX(c);
    if (!V || !qr || !qi || !yr || !yi) return fail(SEM_ERR_ARG, "null field");
    if (apply_direct(c, sizeof(float), V, qr, qi, yr, yi)) {
        // the pipelined kernel sums the side pairs inside its batches; the
        // ring pass then assembles the pairs across batches and the corners
        const bool bulk = c->apply_pipeline && aligned16(V) && aligned16(qr) && aligned16(qi);
        if (bulk) {
            SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
                return launch_apply_bulk<decltype(nv)::value>(c->dm, OP_RES, true, V, alpha, qr, qi, yr, yi, true,
                                                              true, c->apply_pipeline == 2, timeout_ns(c),
                                                              c->stream);
            }));
        } else {
            SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
                return launch_apply<decltype(nv)::value>(c->dm, OP_RES, true, V, alpha, qr, qi, yr, yi, true,
                                                         c->stream);
            }));
        }
        SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
            return launch_ring<decltype(nv)::value>(c->dm, true, DSS_MASK, yr, yi, bulk, c->stream);
        }));
        c->stats.fp32_applies++;
        return SEM_OK;
    }
    float* Y = nullptr;
    int s = wsget(c, "apply_Yf", 2 * c->n, &Y);
    if (s) return s;
    float* Y1 = Y + c->n;
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
        return launch_apply<decltype(nv)::value>(c->dm, OP_RES, true, V, alpha, qr, qi, Y, Y1, true, c->stream);
    }));
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
        return launch_dss<decltype(nv)::value>(c->dm, true, DSS_MASK, 1.0, Y, yr, c->stream);
    }));
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
        return launch_dss<decltype(nv)::value>(c->dm, true, DSS_MASK, 1.0, Y1, yi, c->stream);
    }));
    c->stats.fp32_applies++;
    return SEM_OK;
}

// ------------------------------------------------------ C ABI: Krylov solvers
static int krylov_work(sem_ctx* c, int nc, KrylovWork<double>* w, GridSync** sync, SolveOut** out)
{
    const size_t v = (size_t)nc * c->n;
    const char* ln[3] = {"kr_L0", "kr_L1", "kr_L2"};
    const char* wn[3] = {"kr_W0", "kr_W1", "kr_W2"};
    const char* yn[2] = {"kr_Y0", "kr_Y1"};
    int s = 0;
    for (int k = 0; k < 3; ++k) {
        if ((s = wsget(c, ln[k], v, &w->L[k]))) return s;
        if ((s = wsget(c, wn[k], v, &w->W[k]))) return s;
    }
    for (int k = 0; k < 2; ++k)
        if ((s = wsget(c, yn[k], v, &w->Y[k]))) return s;
    if ((s = wsget(c, "kr_part", 2 * 152 * 64, &w->partials))) return s;
    if ((s = wsget(c, "kr_sync", 1, sync))) return s;
    if ((s = wsget(c, "kr_out", 1, out))) return s;
    return SEM_OK;
}

static int finish_solve(sem_ctx* c, SolveOut* out, GridSync* sync, sem_solver_results* res)
{
    SEM_CUDA(cudaMemcpyAsync(c->h_out, out, sizeof(SolveOut), cudaMemcpyDeviceToHost, c->stream));
    SEM_CUDA(cudaMemcpyAsync(c->h_sync, sync, sizeof(GridSync), cudaMemcpyDeviceToHost, c->stream));
    SEM_CUDA(cudaStreamSynchronize(c->stream));
    if (c->h_sync->err) return fail(SEM_ERR_DEVICE_WAIT, "a grid barrier timed out");
    int s = check_dev_err(c);
    if (s) return s;
    if (c->profile) {
        float ms = 0.f;
        SEM_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
        c->stats.solver_kernel_ms += ms;
    }
    res->success = c->h_out->success;
    res->n_iter = c->h_out->n_iter;
    res->residual = c->h_out->residual;
    c->stats.krylov_iterations += res->n_iter;
    return SEM_OK;
}

// FP64 refinement around an FP32 inner MINRES (SEM_PREC_MIXED)
static int run_mixed(sem_ctx* c, int op, const double* pot, double alpha, double* const x[2],
                     const double* const b[2], int maxit, double tol, int x_is_zero,
                     sem_solver_results* res, int* sweeps, int rel_to_b)
{
    const int nc = (op == OP_RES) ? 2 : 1;
    const size_t v = (size_t)nc * c->n;
    KrylovWork<float> w{};
    const char* ln[3] = {"k32_L0", "k32_L1", "k32_L2"};
    const char* wn[3] = {"k32_W0", "k32_W1", "k32_W2"};
    const char* yn[2] = {"k32_Y0", "k32_Y1"};
    int s = 0;
    for (int k = 0; k < 3; ++k)
        if ((s = wsget(c, ln[k], v, &w.L[k])) || (s = wsget(c, wn[k], v, &w.W[k]))) return s;
    for (int k = 0; k < 2; ++k)
        if ((s = wsget(c, yn[k], v, &w.Y[k]))) return s;
    GridSync* sync = nullptr;
    SolveOut* out = nullptr;
    double *r64 = nullptr, *Y64 = nullptr;
    float *x32 = nullptr, *pot32 = nullptr;
    if ((s = wsget(c, "kr_part", 2 * 152 * 64, &w.partials)) || (s = wsget(c, "kr_sync", 1, &sync)) ||
        (s = wsget(c, "kr_out", 1, &out)) || (s = wsget(c, "mx_r64", v, &r64)) ||
        (s = wsget(c, "mx_Y64", v, &Y64)) || (s = wsget(c, "mx_x32", v, &x32)) ||
        (s = wsget(c, "mx_pot32", c->n, &pot32)))
        return s;
    k_to_f32<<<grid_1d(c->n), 256, 0, c->stream>>>(c->n, pot, pot32);
    c->stats.kernel_launches++;
    SEM_CUDA(cudaGetLastError());
    MixedArgs mx{};
    mx.inner_tol = c->inner_tol;
    mx.max_sweeps = c->max_refine;
    mx.inner_maxit = maxit;
    for (int q = 0; q < 2; ++q) {
        mx.r64[q] = r64 + (size_t)q * c->n;
        mx.Y64[q] = Y64 + (size_t)q * c->n;
        mx.x32[q] = x32 + (size_t)q * c->n;
    }
    mx.pot32 = pot32;
    mx.pinv32 = nullptr;
    mx.fused = c->inner_fused;
    mx.outer_scale = c->outer_scale;
    mx.adaptive = c->adaptive_inner;
    if (c->inner_fused) {
        if ((s = wsget(c, "k32_AZ", v, &w.AZ)) || (s = wsget(c, "k32_Y3", v, &w.Y3))) return s;
    }
    if (c->precond == SEM_PRECOND_FDM && op == OP_RES) {
        if ((s = wsget(c, "k32_Z0", v, &w.Z[0])) || (s = wsget(c, "k32_Z1", v, &w.Z[1])) ||
            (s = wsget(c, "k32_Y3", v, &w.Y3)))
            return s;
        mx.fdm = 1;
        mx.fused = 0;
    } else if (c->precond) {
        float* pinv = nullptr;
        if ((s = wsget(c, "mx_pinv32", c->n, &pinv))) return s;
        k_prec<<<grid_1d(c->n), 256, 0, c->stream>>>(c->n, op, alpha, c->dm.mdiag, c->dm.kdiag, pot, pinv);
        c->stats.kernel_launches++;
        SEM_CUDA(cudaGetLastError());
        mx.pinv32 = pinv;
    }
    int grid = 0, kmax = 1, rst = 0;
    size_t smem = 0;
    bool resident = false;
    if (mx.fdm && c->resident)
        dispatch_resident(c->N, [&](auto nv) {
            resident = resident_plan<decltype(nv)::value>(c->E, c->sms, kResidentSmemBudget, &grid, &rst, &kmax,
                                                          &smem);
        });
    if (!resident)
        dispatch_n(c->N, [&](auto nv) {
            grid = solver_plan<decltype(nv)::value>(op, true, c->E, c->sms, kSolverSmemBudget, &kmax, &smem);
            return cudaSuccess;
        });
    if (grid <= 0) return fail(SEM_ERR_CUDA, "could not size the cooperative grid");
    unsigned long long *slots = nullptr, *xa = nullptr, *xb = nullptr;
    if (resident) {
        const size_t words = 2 * (size_t)grid * RESIDENT_SLOT_STRIDE;
        if ((s = wsget(c, "res_slots", words, &slots)) || (s = wsget(c, "res_xa", 2 * (size_t)c->n, &xa)) ||
            (s = wsget(c, "res_xb", 2 * (size_t)c->n, &xb)))
            return s;
        SEM_CUDA(cudaMemsetAsync(slots, 0, words * sizeof(unsigned long long), c->stream));
        SEM_CUDA(cudaMemsetAsync(xa, 0, 2 * (size_t)c->n * sizeof(unsigned long long), c->stream));
        SEM_CUDA(cudaMemsetAsync(xb, 0, 2 * (size_t)c->n * sizeof(unsigned long long), c->stream));
    }
    SolveArgs a{};
    a.kmax = kmax;
    a.op = op;
    a.nc = nc;
    a.pot = pot;
    a.alpha = alpha;
    a.b[0] = b[0];
    a.b[1] = nc == 2 ? b[1] : nullptr;
    a.x[0] = x[0];
    a.x[1] = nc == 2 ? x[1] : nullptr;
    a.maxit = maxit;
    a.tol = tol;
    a.x_is_zero = x_is_zero;
    a.rel_to_b = rel_to_b;
    a.timeout_ns = (long long)(c->timeout_ms * 1e6);
    a.sync = sync;
    a.out = out;
    SEM_CUDA(cudaMemsetAsync(sync, 0, sizeof(GridSync), c->stream));
    SEM_CUDA(cudaMemsetAsync(out, 0, sizeof(SolveOut), c->stream));
    if (c->profile) SEM_CUDA(cudaEventRecord(c->ev[0], c->stream));
    cudaError_t e = cudaSuccess;
    if (resident)
        dispatch_resident(c->N, [&](auto nv) {
            e = launch_resident<decltype(nv)::value>(c->dm, a, w, mx, c->D32_host.data(), c->S32_host.data(), rst,
                                                     slots, xa, xb, grid, smem, c->stream);
        });
    else
        e = dispatch_n(c->N, [&](auto nv) {
            return launch_solver<decltype(nv)::value>(c->dm, a, &w, &mx, grid, smem, c->stream);
        });
    if (e != cudaSuccess) return fail(SEM_ERR_CUDA, std::string("cooperative launch: ") + cudaGetErrorString(e));
    if (c->profile) SEM_CUDA(cudaEventRecord(c->ev[1], c->stream));
    c->stats.kernel_launches++;
    c->stats.solver_launches++;
    if (resident) c->stats.resident_launches++;
    if ((s = finish_solve(c, out, sync, res))) return s;
    *sweeps = c->h_out->sweeps;
    c->stats.solver_iterations_fp32 += res->n_iter;
    c->stats.fp32_applies += res->n_iter + *sweeps;
    c->stats.fp64_applies += *sweeps + 1;
    return SEM_OK;
}

static int run_krylov(sem_ctx* c, int op, const double* pot, double alpha, double* const x[2],
                      const double* const b[2], int maxit, double tol, int x_is_zero,
                      sem_solver_results* res, int* sweeps = nullptr, int rel_to_b = 0)
{
    if (sweeps) *sweeps = 1;
    if (c->prec == SEM_PREC_MIXED && op != OP_LAPLACE) {
        int sw = 0;
        int s = run_mixed(c, op, pot, alpha, x, b, maxit, tol, x_is_zero, res, &sw, rel_to_b);
        if (sweeps) *sweeps = sw;
        return s;
    }
    const int nc = (op == OP_RES) ? 2 : 1;
    KrylovWork<double> w{};
    GridSync* sync = nullptr;
    SolveOut* out = nullptr;
    int s = krylov_work(c, nc, &w, &sync, &out);
    if (s) return s;
    int grid = 0, kmax = 1;
    size_t smem = 0;
    dispatch_n(c->N, [&](auto nv) {
        grid = solver_plan<decltype(nv)::value>(op, false, c->E, c->sms, kSolverSmemBudget, &kmax, &smem);
        return cudaSuccess;
    });
    if (grid <= 0) return fail(SEM_ERR_CUDA, "could not size the cooperative grid");
    SolveArgs a{};
    a.kmax = kmax;
    a.op = op;
    a.nc = nc;
    a.pot = pot;
    a.alpha = alpha;
    a.b[0] = b[0];
    a.b[1] = nc == 2 ? b[1] : nullptr;
    a.x[0] = x[0];
    a.x[1] = nc == 2 ? x[1] : nullptr;
    a.maxit = maxit;
    a.tol = tol;
    a.x_is_zero = x_is_zero;
    a.timeout_ns = (long long)(c->timeout_ms * 1e6);
    a.sync = sync;
    a.out = out;
    SEM_CUDA(cudaMemsetAsync(sync, 0, sizeof(GridSync), c->stream));
    SEM_CUDA(cudaMemsetAsync(out, 0, sizeof(SolveOut), c->stream));
    if (c->profile) SEM_CUDA(cudaEventRecord(c->ev[0], c->stream));
    cudaError_t e = dispatch_n(c->N, [&](auto nv) {
        return launch_solver<decltype(nv)::value>(c->dm, a, &w, nullptr, grid, smem, c->stream);
    });
    if (e != cudaSuccess) return fail(SEM_ERR_CUDA, std::string("cooperative launch: ") + cudaGetErrorString(e));
    if (c->profile) SEM_CUDA(cudaEventRecord(c->ev[1], c->stream));
    c->stats.kernel_launches++;
    c->stats.solver_launches++;
    if ((s = finish_solve(c, out, sync, res))) return s;
    c->stats.solver_iterations_fp64 += res->n_iter;
    c->stats.fp64_applies += res->n_iter + 1 + (x_is_zero ? 0 : 1);
    return SEM_OK;
}

extern "C" int sem_minres_schro(sem_ctx* c, const double* V, double alpha, double* xr, double* xi,
                                const double* br, const double* bi, int maxit, double tol,
                                int x_is_zero, sem_solver_results* res)
{
    SEM_CHECK_CTX(c);
    if (!V || !xr || !xi || !br || !bi || !res) return fail(SEM_ERR_ARG, "null argument");
    double* x[2] = {xr, xi};
    const double* b[2] = {br, bi};
    return run_krylov(c, OP_RES, V, alpha, x, b, maxit, tol, x_is_zero, res);
}

extern "C" int sem_minres_helmholtz(sem_ctx* c, const double* cf, double* x, const double* b,
                                    int maxit, double tol, int x_is_zero, sem_solver_results* res)
{
    SEM_CHECK_CTX(c);
    if (!cf || !x || !b || !res) return fail(SEM_ERR_ARG, "null argument");
    double* xx[2] = {x, nullptr};
    const double* bb[2] = {b, nullptr};
    return run_krylov(c, OP_HELM, cf, 0.0, xx, bb, maxit, tol, x_is_zero, res);
}

extern "C" int sem_pcg_laplace(sem_ctx* c, double* x, const double* b, int max_iter, double tol,
                               int x_is_zero, sem_solver_results* res)
{
    SEM_CHECK_CTX(c);
    if (!x || !b || !res) return fail(SEM_ERR_ARG, "null argument");
    double* xx[2] = {x, nullptr};
    const double* bb[2] = {b, nullptr};
    return run_krylov(c, OP_LAPLACE, nullptr, 0.0, xx, bb, max_iter, tol, x_is_zero, res);
}

// ------------------------------------------------------------ C ABI: drivers
// stage a caller field on the device: returns a device pointer (the caller's
// own when it already is one)
static int stage_in(sem_ctx* c, const char* name, const double* src, size_t count, const double** out,
                    bool* was_host)
{
    *was_host = !is_device_ptr(src);
    if (!*was_host) {
        *out = src;
        return SEM_OK;
    }
    double* d = nullptr;
    int s = wsget(c, name, count, &d);
    if (s) return s;
    SEM_CUDA(cudaMemcpyAsync(d, src, sizeof(double) * count, cudaMemcpyHostToDevice, c->stream));
    *out = d;
    return SEM_OK;
}

extern "C" int sem_poisson(sem_ctx* c, double* u, const double* f, int max_iter, double tol,
                           sem_solver_results* res)
{
    SEM_CHECK_CTX(c);
    if (!u || !f || !res) return fail(SEM_ERR_ARG, "null argument");
    bool uh = false, fh = false;
    const double* fd = nullptr;
    const double* ud0 = nullptr;
    int s = 0;
    if ((s = stage_in(c, "drv_f", f, c->n, &fd, &fh))) return s;
    if ((s = stage_in(c, "drv_u", u, c->n, &ud0, &uh))) return s;
    double* ud = const_cast<double*>(ud0);
    double* b = nullptr;
    if ((s = wsget(c, "drv_b", c->n, &b))) return s;
    if ((s = sem_gproj(c, fd, b))) return s;  // poisson.hpp:20
    if ((s = sem_pcg_laplace(c, ud, b, max_iter, tol, 0, res))) return s;
    if (uh) {
        SEM_CUDA(cudaMemcpyAsync(u, ud, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
        SEM_CUDA(cudaStreamSynchronize(c->stream));
    }
    return SEM_OK;
}

extern "C" int sem_helmholtz(sem_ctx* c, double* u, const double* cf, const double* f, int max_iter,
                             double tol, sem_solver_results* res)
{
    SEM_CHECK_CTX(c);
    if (!u || !cf || !f || !res) return fail(SEM_ERR_ARG, "null argument");
    bool uh = false, fh = false, ch = false;
    const double *fd = nullptr, *cd = nullptr, *ud0 = nullptr;
    int s = 0;
    if ((s = stage_in(c, "drv_f", f, c->n, &fd, &fh))) return s;
    if ((s = stage_in(c, "drv_c", cf, c->n, &cd, &ch))) return s;
    if ((s = stage_in(c, "drv_u", u, c->n, &ud0, &uh))) return s;
    double* ud = const_cast<double*>(ud0);
    double* b = nullptr;
    if ((s = wsget(c, "drv_b", c->n, &b))) return s;
    if ((s = sem_gproj(c, fd, b))) return s;  // helmholtz.hpp:21
    if ((s = sem_minres_helmholtz(c, cd, ud, b, max_iter, tol, 0, res))) return s;
    if (uh) {
        SEM_CUDA(cudaMemcpyAsync(u, ud, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
        SEM_CUDA(cudaStreamSynchronize(c->stream));
    }
    return SEM_OK;
}

// --------------------------------------------- boundary data (no counterpart)
// Element-local field built from the boundary data g (host or device):
// Dirichlet context, g is an element-local field and the result the lifting
// u_D (g at every copy of a boundary node, 0 elsewhere); Neumann context, g
// holds du/dn per element side node ([E][4][N], side s as in DevMesh::flags,
// node k along the side in the element's own direction) and the result is
// the boundary integral of g against each basis function, w_k (L/2) g_k at
// node k of every boundary side of length L (GLL quadrature on the straight
// side), a corner copy collecting the terms of each of its element's
// boundary sides that meet there.  Written to dev.
static int bc_field(sem_ctx* c, const double* g, double* dev)
{
    const int N = c->N, NN = N * N;
    const bool neumann = (c->flags & SEM_FLAG_NEUMANN) != 0;
    const size_t ng = neumann ? (size_t)c->E * 4 * N : (size_t)c->n;
    std::vector<double> gh(ng), F((size_t)c->n, 0.0);
    if (is_device_ptr(g)) {
        SEM_CUDA(cudaMemcpyAsync(gh.data(), g, sizeof(double) * ng, cudaMemcpyDeviceToHost, c->stream));
        SEM_CUDA(cudaStreamSynchronize(c->stream));
    } else {
        std::copy(g, g + ng, gh.begin());
    }
    static const int ca[] = {0, 1, 3, 0}, cb[] = {1, 2, 2, 3};  // corners of side s, k = 0 at ca
    auto flat_of = [&](int e, int s, int k) -> size_t {
        const size_t b = (size_t)e * NN;
        switch (s) {
            case 0: return b + k;
            case 1: return b + (N - 1) + (size_t)k * N;
            case 2: return b + k + (size_t)(N - 1) * N;
            default: return b + (size_t)k * N;
        }
    };
    for (int e = 0; e < c->E; ++e) {
        const int fe = c->fl_host[e];
        for (int sd = 0; sd < 4; ++sd) {
            if (!(fe & ((neumann ? 65536 : 16) << sd))) continue;
            if (!neumann) {
                for (int k = 0; k < N; ++k) F[flat_of(e, sd, k)] = gh[flat_of(e, sd, k)];
                continue;
            }
            const int a = c->elements[4 * (size_t)e + ca[sd]], b = c->elements[4 * (size_t)e + cb[sd]];
            const double half = 0.5 * std::hypot(c->coords[2 * (size_t)b] - c->coords[2 * (size_t)a],
                                                 c->coords[2 * (size_t)b + 1] - c->coords[2 * (size_t)a + 1]);
            for (int k = 0; k < N; ++k) F[flat_of(e, sd, k)] += c->w[k] * half * gh[((size_t)e * 4 + sd) * N + k];
        }
        if (!neumann) {  // copies of boundary corner nodes whose sides are interior
            for (int cc = 0; cc < 4; ++cc)
                if (fe & (4096 << cc)) {
                    const size_t f = (size_t)e * NN + (cc == 1 || cc == 2 ? N - 1 : 0) +
                                     (cc >= 2 ? (size_t)(N - 1) * N : 0);
                    F[f] = gh[f];
                }
        }
    }
    SEM_CUDA(cudaMemcpyAsync(dev, F.data(), sizeof(double) * c->n, cudaMemcpyHostToDevice, c->stream));
    SEM_CUDA(cudaStreamSynchronize(c->stream));
    return SEM_OK;
}

static int bc_solve(sem_ctx* c, bool helm, double* u, const double* cf, const double* f, const double* g,
                    int max_iter, double tol, sem_solver_results* res)
{
    SEM_CHECK_CTX(c);
    if (!u || !f || !g || !res || (helm && !cf)) return fail(SEM_ERR_ARG, "null argument");
    bool uh = false, fh = false, ch = false;
    const double *fd = nullptr, *cd = nullptr, *ud0 = nullptr;
    int s = 0;
    if ((s = stage_in(c, "drv_f", f, c->n, &fd, &fh))) return s;
    if (helm && (s = stage_in(c, "drv_c", cf, c->n, &cd, &ch))) return s;
    if ((s = stage_in(c, "drv_u", u, c->n, &ud0, &uh))) return s;
    double* ud = const_cast<double*>(ud0);
    double *b = nullptr, *F = nullptr, *T = nullptr;
    if ((s = wsget(c, "drv_b", c->n, &b)) || (s = wsget(c, "bc_F", c->n, &F)) || (s = wsget(c, "bc_T", c->n, &T)))
        return s;
    if ((s = bc_field(c, g, F))) return s;
    if ((s = sem_gproj(c, fd, b))) return s;
    const bool neumann = (c->flags & SEM_FLAG_NEUMANN) != 0;
    if (!neumann) {  // b -= A u_D (masked rows: the interior equations)
        if ((s = apply_galerkin(c, helm ? OP_HELM : OP_LAPLACE, cd, 0.0, F, nullptr, T, nullptr))) return s;
    } else {  // b += the assembled boundary integral
        SEM_CUDA(cudaMemcpyAsync(T, F, sizeof(double) * c->n, cudaMemcpyDeviceToDevice, c->stream));
        if ((s = sem_global_sum(c, T)) || (s = sem_mask(c, T))) return s;
    }
    if ((s = sem_vec_axpby(c, c->n, 1.0, b, neumann ? 1.0 : -1.0, T, b))) return s;
    if ((s = sem_mask(c, ud))) return s;  // the guess of the interior part
    if (helm) {
        if ((s = sem_minres_helmholtz(c, cd, ud, b, max_iter, tol, 0, res))) return s;
    } else {
        if ((s = sem_pcg_laplace(c, ud, b, max_iter, tol, 0, res))) return s;
    }
    if ((s = sem_unmask(c, ud))) return s;
    if (!neumann && (s = sem_vec_axpby(c, c->n, 1.0, ud, 1.0, F, ud))) return s;  // u = u0 + u_D
    if (uh) {
        SEM_CUDA(cudaMemcpyAsync(u, ud, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
        SEM_CUDA(cudaStreamSynchronize(c->stream));
    }
    return SEM_OK;
}

extern "C" int sem_poisson_bc(sem_ctx* c, double* u, const double* f, const double* g, int max_iter, double tol,
                              sem_solver_results* res)
{
    return bc_solve(c, false, u, nullptr, f, g, max_iter, tol, res);
}

extern "C" int sem_helmholtz_bc(sem_ctx* c, double* u, const double* cf, const double* f, const double* g,
                                int max_iter, double tol, sem_solver_results* res)
{
    return bc_solve(c, true, u, cf, f, g, max_iter, tol, res);
}

// state shared by the three Schroedinger drivers
struct SchroRun {
    sem_ctx* c;
    double* psi_re;
    double* psi_im;
    bool host;
    const double* V;  // device
    double* P[2];     // two-plane state ping-pong
    int cur;
    long long n;
};

static int schro_begin(sem_ctx* c, double* psi_re, double* psi_im, const double* V, SchroRun* r)
{
    r->c = c;
    r->psi_re = psi_re;
    r->psi_im = psi_im;
    r->n = c->n;
    r->cur = 0;
    r->host = !is_device_ptr(psi_re);
    bool vh = false;
    int s = 0;
    if ((s = stage_in(c, "drv_V", V, c->n, &r->V, &vh))) return s;
    if ((s = wsget(c, "drv_P0", 2 * c->n, &r->P[0]))) return s;
    if ((s = wsget(c, "drv_P1", 2 * c->n, &r->P[1]))) return s;
    const cudaMemcpyKind k = r->host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    SEM_CUDA(cudaMemcpyAsync(r->P[0], psi_re, sizeof(double) * c->n, k, c->stream));
    SEM_CUDA(cudaMemcpyAsync(r->P[0] + c->n, psi_im, sizeof(double) * c->n, k, c->stream));
    c->stats.steps_taken = 0;
    return SEM_OK;
}

static int schro_publish(SchroRun* r)
{
    sem_ctx* c = r->c;
    const cudaMemcpyKind k = r->host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    SEM_CUDA(cudaMemcpyAsync(r->psi_re, r->P[r->cur], sizeof(double) * c->n, k, c->stream));
    SEM_CUDA(cudaMemcpyAsync(r->psi_im, r->P[r->cur] + c->n, sizeof(double) * c->n, k, c->stream));
    SEM_CUDA(cudaStreamSynchronize(c->stream));
    return check_dev_err(c);
}

// b = dt * f(p + sum a_l z_l), masked (schrodinger.hpp:221,229,378,386)
static int schro_rhs(SchroRun* r, double dt, const ZList& zl, double* b)
{
    sem_ctx* c = r->c;
    double* Y = nullptr;
    int s = wsget(c, "apply_Y", 2 * c->n, &Y);
    if (s) return s;
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
        return launch_combo_f<decltype(nv)::value>(c->dm, r->V, r->P[r->cur], zl, Y, c->stream);
    }));
    for (int q = 0; q < 2; ++q)
        SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
            return launch_dss<decltype(nv)::value>(c->dm, false, DSS_MASK, dt, Y + q * c->n, b + q * c->n, c->stream);
        }));
    c->stats.fp64_applies++;
    return SEM_OK;
}

static int schro_stage_solve(SchroRun* r, double alpha, const double* b, double* z, int max_iter,
                             double tol, int x_is_zero, sem_solver_results* res, int* sweeps)
{
    sem_ctx* c = r->c;
    double* x[2] = {z, z + c->n};
    const double* bb[2] = {b, b + c->n};
    // a warm-started stage is judged relative to |b|, which is the
    // reference's test (relative to |r_0| = |b|) for the zero start
    return run_krylov(c, OP_RES, r->V, alpha, x, bb, max_iter, tol, x_is_zero, res, sweeps, !x_is_zero);
}

// ------------------------------------------------------ learned stage guess
static int launch_learn_op(sem_ctx* c, const LearnArgs& a)
{
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) { return launch_learn<decltype(nv)::value>(c->dm, a, c->stream); }));
    return SEM_OK;
}

// r = b - A z (continuous format, two planes) for a guess z
static int guess_residual(sem_ctx* c, const double* V, double alpha, const double* b, const double* z, double* r)
{
    double* Y = nullptr;
    int s = wsget(c, "lr_Y", 2 * c->n, &Y);
    if (s) return s;
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
        return launch_apply<decltype(nv)::value>(c->dm, OP_RES, false, V, alpha, z, z + c->n, Y, Y + c->n, true,
                                                 c->stream);
    }));
    LearnArgs a{};
    a.what = LEARN_RESID;
    a.b = b;
    a.Y = Y;
    a.r = r;
    c->stats.fp64_applies++;
    return launch_learn_op(c, a);
}

// (a.a, a.b, b.b) of two-plane vectors, owner-weighted, one synchronisation
static int dots3(sem_ctx* c, const double* a, const double* b, double* aa, double* ab, double* bbv)
{
    double* part = nullptr;
    int s = wsget(c, "dot_part", 152 * 64, &part);
    if (s) return s;
    int used = 0;
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
        return launch_dot3<decltype(nv)::value>(c->dm, a, b, part, 152 * 64 / 3, &used, c->stream);
    }));
    SEM_CUDA(cudaMemcpyAsync(c->h_part, part, sizeof(double) * 3 * used, cudaMemcpyDeviceToHost, c->stream));
    SEM_CUDA(cudaStreamSynchronize(c->stream));
    double s0 = 0, s1 = 0, s2 = 0;
    for (int i = 0; i < used; ++i) {
        s0 += c->h_part[3 * i];
        s1 += c->h_part[3 * i + 1];
        s2 += c->h_part[3 * i + 2];
    }
    if (aa) *aa = s0;
    if (ab) *ab = s1;
    if (bbv) *bbv = s2;
    return SEM_OK;
}

// Build the per-element features of the extrapolated guess z (its scaled
// residual, alpha V, mass / alpha); with `use`, let the network predict a
// correction and move z along it by the residual-minimising step (none when
// no positive step lowers the FP64 residual: the extrapolation stays the
// fallback).  *zext receives a copy of the extrapolated guess (the base the
// training targets are measured from).
static int learned_guess(sem_ctx* c, const double* V, double alpha, const double* b, double* z, bool use,
                         double** zext, const double* rbase)
{
    const int NN = c->N * c->N;
    double *r = nullptr, *zx = nullptr;
    void* x = nullptr;
    float* sig = nullptr;
    int s = 0;
    if ((s = wsget(c, "lr_r", 2 * c->n, &r)) || (s = wsget(c, "lr_zext", 2 * c->n, &zx)) ||
        (s = wsbuf(c, "lr_x", (size_t)c->E * 4 * NN * 2, &x)) || (s = wsget(c, "lr_sig", c->E, &sig)))
        return s;
    SEM_CUDA(cudaMemcpyAsync(zx, z, sizeof(double) * 2 * c->n, cudaMemcpyDeviceToDevice, c->stream));
    *zext = zx;
    if (rbase)  // the base guess's residual is known (projection): continuous copy
        SEM_CUDA(cudaMemcpyAsync(r, rbase, sizeof(double) * 2 * c->n, cudaMemcpyDeviceToDevice, c->stream));
    else if ((s = guess_residual(c, V, alpha, b, zx, r)))
        return s;
    // per-element scale floor: 1e-6 of the residual's RMS over all copies.
    // A prediction takes |r|^2 from the previous learned guess of the run
    // (the floor only keeps round-off out of the features); the first one,
    // and every training sample, reads it back for this residual
    double n_ext = c->lr_nrm2;
    if (!use || !(n_ext > 0)) {
        if ((s = dots3(c, r, r, &n_ext, nullptr, nullptr))) return s;
        c->lr_nrm2 = n_ext;
    }
    LearnArgs a{};
    a.what = LEARN_FEATURES;
    a.r = r;
    a.V = V;
    a.alpha = alpha;
    a.rho_floor = std::max(1e-6 * std::sqrt(n_ext / (2.0 * (double)c->n)), 1e-300);
    a.x = x;
    a.sigma = sig;
    if ((s = launch_learn_op(c, a))) return s;
    if (!use) return SEM_OK;
    float* delta = nullptr;
    double* zl = nullptr;
    if ((s = wsget(c, "lr_delta", (size_t)c->E * 2 * NN, &delta)) || (s = wsget(c, "lr_zl", 2 * c->n, &zl)))
        return s;
    const long long fl0 = learner_forward_launches(c->learner);
    if ((s = sem_learner_set_stream(c->learner, c->stream)) || (s = sem_learner_forward(c->learner, c->E, x, delta)))
        return s;
    c->stats.kernel_launches += learner_forward_launches(c->learner) - fl0;
    LearnArgs k{};
    k.what = LEARN_CORRECT;
    k.zg = zx;
    k.sigma = sig;
    k.delta = delta;
    k.zo = zl;
    if ((s = launch_learn_op(c, k))) return s;
    // minimal residual along the predicted correction d = z_l - z_ext:
    // r(theta) = r_ext - theta A d, so theta = r_ext.Ad / |Ad|^2 and
    // |r(theta)| <= |r_ext|.  A d only sets the step length, so it is
    // applied in FP32; the stage solve judges the guess on its true FP64
    // residual.  The step is taken on the device (no read-back before the
    // solve); its statistics are collected after it (learned_collect)
    float *d32 = nullptr, *ad32 = nullptr, *v32 = nullptr;
    if ((s = wsget(c, "lr_d32", 2 * c->n, &d32)) || (s = wsget(c, "lr_ad32", 2 * c->n, &ad32)) ||
        (s = wsget(c, "lr_v32", c->n, &v32)))
        return s;
    k_diff_f32<<<grid_1d(2 * c->n), 256, 0, c->stream>>>(2 * c->n, zl, zx, d32);
    SEM_CUDA(cudaGetLastError());
    k_to_f32<<<grid_1d(c->n), 256, 0, c->stream>>>(c->n, V, v32);
    SEM_CUDA(cudaGetLastError());
    c->stats.kernel_launches += 2;
    if ((s = sem_apply_schro_res_f32(c, v32, (float)alpha, d32, d32 + c->n, ad32, ad32 + c->n))) return s;
    double* part = nullptr;
    double* dst = nullptr;
    if ((s = wsget(c, "dot_part", 152 * 64, &part)) || (s = wsget(c, "lr_stat", 4, &dst))) return s;
    int used = 0;
    SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
        return launch_dot3_f32<decltype(nv)::value>(c->dm, r, ad32, part, 152 * 64 / 3, &used, c->stream);
    }));
    k_learn_theta<<<1, 256, 0, c->stream>>>(part, used, c->learned_step == 1 ? 1 : 0, dst);
    SEM_CUDA(cudaGetLastError());
    k_learn_step<<<grid_1d(2 * c->n), 256, 0, c->stream>>>(2 * c->n, zx, zl, dst, z);
    SEM_CUDA(cudaGetLastError());
    c->stats.kernel_launches += 2;
    SEM_CUDA(cudaMemcpyAsync(c->h_lstat, dst, sizeof(double) * 4, cudaMemcpyDeviceToHost, c->stream));
    c->stats.learned_guesses++;
    c->lr_pending = true;
    return SEM_OK;
}

// statistics of the last learned step, once the stream has passed it (the
// stage solve's read-back synchronises the stream)
static int learned_collect(sem_ctx* c)
{
    if (!c->lr_pending) return SEM_OK;
    SEM_CUDA(cudaStreamSynchronize(c->stream));  // a no-op after the solve's read-back
    const double* h = c->h_lstat;
    c->lr_nrm2 = h[0];
    c->stats.last_guess_theta = h[1];
    c->stats.last_guess_residual_ratio = h[2];
    c->stats.learned_ratio_sum += h[2];
    if (h[3] != 0.0) c->stats.learned_accepted++;
    c->lr_pending = false;
    return SEM_OK;
}

// append (features, (z - zext)/sigma) of every element to the dataset
static int record_sample(sem_ctx* c, const double* z, const double* zext)
{
    const int NN = c->N * c->N;
    if (c->ds_rows + c->E > c->ds_cap) return SEM_OK;  // full: keep the first samples
    void* x = nullptr;
    float *sig = nullptr, *t = nullptr;
    int s = 0;
    if ((s = wsbuf(c, "lr_x", (size_t)c->E * 4 * NN * 2, &x)) || (s = wsget(c, "lr_sig", c->E, &sig)) ||
        (s = wsget(c, "lr_t", (size_t)c->E * 2 * NN, &t)))
        return s;
    LearnArgs a{};
    a.what = LEARN_TARGETS;
    a.z = z;
    a.zg = zext;
    a.sigma = sig;
    a.t = t;
    if ((s = launch_learn_op(c, a))) return s;
    void* dX = nullptr;
    float* dT = nullptr;
    if ((s = wsbuf(c, "ds_X", (size_t)c->ds_cap * 4 * NN * 2, &dX)) ||
        (s = wsget(c, "ds_T", (size_t)c->ds_cap * 2 * NN, &dT)))
        return s;
    SEM_CUDA(cudaMemcpyAsync((char*)dX + (size_t)c->ds_rows * 4 * NN * 2, x, (size_t)c->E * 4 * NN * 2,
                             cudaMemcpyDeviceToDevice, c->stream));
    SEM_CUDA(cudaMemcpyAsync(dT + (size_t)c->ds_rows * 2 * NN, t, (size_t)c->E * 2 * NN * sizeof(float),
                             cudaMemcpyDeviceToDevice, c->stream));
    c->ds_rows += c->E;
    return SEM_OK;
}

extern "C" int sem_ctx_set_learner(sem_ctx* c, sem_learner* L)
{
    SEM_CHECK_CTX(c);
    if (L) {
        int din = 0, dout = 0;
        int s = sem_learner_shape(L, &din, nullptr, &dout);
        if (s) return s;
        if (din != 4 * c->N * c->N || dout != 2 * c->N * c->N)
            return fail(SEM_ERR_ARG, "learner shape must be 4 N^2 -> 2 N^2 for this mesh");
    }
    c->learner = L;
    c->lr_nrm2 = -1.0;
    return SEM_OK;
}

extern "C" int sem_ctx_record(sem_ctx* c, long long capacity_rows)
{
    SEM_CHECK_CTX(c);
    if (capacity_rows < 0) return fail(SEM_ERR_ARG, "negative capacity");
    c->ds_cap = capacity_rows;
    c->ds_rows = 0;
    return SEM_OK;
}

extern "C" int sem_ctx_dataset(sem_ctx* c, void** X, float** T, long long* rows, int* d_in, int* d_out)
{
    SEM_CHECK_CTX(c);
    const int NN = c->N * c->N;
    if (d_in) *d_in = 4 * NN;
    if (d_out) *d_out = 2 * NN;
    if (rows) *rows = c->ds_rows;
    void* dX = nullptr;
    float* dT = nullptr;
    if (c->ds_cap > 0) {
        int s = 0;
        if ((s = wsbuf(c, "ds_X", (size_t)c->ds_cap * 4 * NN * 2, &dX)) ||
            (s = wsget(c, "ds_T", (size_t)c->ds_cap * 2 * NN, &dT)))
            return s;
    }
    if (X) *X = dX;
    if (T) *T = dT;
    return SEM_OK;
}

// ------------------------------------------------ projection stage guess
// P. F. Fischer, "Projection techniques for iterative solution of Ax = b with
// successive right-hand sides", Comput. Methods Appl. Mech. Engrg. 163
// (1998), in a residual-minimising form for the indefinite stage operator:
// the driver keeps the last proj_k stage solutions z_j with their right-hand
// sides b_j (A z_j = b_j to the solver tolerance: every stage of an SDIRK or
// BDF2 run at fixed dt has the same operator), and a new stage starts from
// x0 = sum_j c_j z_j with c minimising |b - sum_j c_j b_j| (normal equations
// on the Gram matrix of the b_j, Jacobi scaled, directions whose eigenvalue
// is below 1e-13 of the largest dropped).  Slot j of the workspace holds z_j
// (two planes) then b_j (two planes).
static int proj_slots(sem_ctx* c, double** slots)
{
    return wsget(c, "proj_slots", (size_t)c->proj_k * 4 * c->n, slots);
}

// d[j] = b.b_j for every stored slot, *bb = b.b (one pass over the vectors)
static int proj_dots(sem_ctx* c, const double* b, const double* slots, std::vector<double>& d, double* bb)
{
    const long long v = 2 * c->n;
    PtrList L{};
    L.nz = c->proj_count;
    for (int j = 0; j < L.nz; ++j) L.z[j] = slots + (size_t)j * 2 * v + v;
    constexpr int blocks = 256;
    double* part = nullptr;
    int s = wsget(c, "proj_part", (size_t)blocks * (PROJ_MAX + 1), &part);
    if (s) return s;
    k_multidot<<<blocks, 256, 0, c->stream>>>(v, b, L, part);
    c->stats.kernel_launches++;
    SEM_CUDA(cudaGetLastError());
    SEM_CUDA(cudaMemcpyAsync(c->h_part, part, sizeof(double) * blocks * (PROJ_MAX + 1), cudaMemcpyDeviceToHost,
                             c->stream));
    SEM_CUDA(cudaStreamSynchronize(c->stream));
    d.assign(L.nz, 0.0);
    double acc = 0.0;
    for (int q = 0; q < blocks; ++q) {
        const double* row = c->h_part + (size_t)q * (PROJ_MAX + 1);
        for (int j = 0; j < L.nz; ++j) d[j] += row[j];
        acc += row[PROJ_MAX];
    }
    *bb = acc;
    return SEM_OK;
}

// x0 = sum_j c_j z_j from the stored slots; returns the estimated relative
// residual |b - sum c_j b_j| / |b| in *ratio (1 when no basis direction is
// kept, then x0 = 0)
static int proj_guess(sem_ctx* c, const double* slots, const std::vector<double>& d, double bb, double* x0,
                      double* ratio, std::vector<double>* coef)
{
    const int k = c->proj_count;
    const int K = c->proj_k;
    std::vector<double> sc(k), A((size_t)k * k), Q, cf(k, 0.0);
    for (int i = 0; i < k; ++i) {
        const double g = c->proj_G[(size_t)i * K + i];
        sc[i] = g > 0 ? 1.0 / std::sqrt(g) : 0.0;
    }
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) A[(size_t)i * k + j] = sc[i] * c->proj_G[(size_t)i * K + j] * sc[j];
    sym_eig_jacobi(k, A, Q);
    double lmax = 0.0;
    for (int i = 0; i < k; ++i) lmax = std::max(lmax, A[(size_t)i * k + i]);
    for (int m = 0; m < k; ++m) {
        const double lam = A[(size_t)m * k + m];
        if (!(lam > 1e-13 * lmax)) continue;
        double qd = 0.0;
        for (int i = 0; i < k; ++i) qd += Q[(size_t)i * k + m] * sc[i] * d[i];
        for (int i = 0; i < k; ++i) cf[i] += Q[(size_t)i * k + m] * qd / lam;
    }
    double cd = 0.0;
    for (int i = 0; i < k; ++i) {
        cf[i] *= sc[i];
        cd += cf[i] * d[i];
    }
    PtrList L{};
    L.nz = k;
    for (int j = 0; j < k; ++j) {
        L.z[j] = slots + (size_t)j * 4 * c->n;
        L.c[j] = cf[j];
    }
    k_lincomb_n<<<grid_1d(2 * c->n), 256, 0, c->stream>>>(2 * c->n, L, x0);
    c->stats.kernel_launches++;
    SEM_CUDA(cudaGetLastError());
    *ratio = bb > 0 ? std::sqrt(std::max(0.0, bb - cd) / bb) : 1.0;
    if (coef) *coef = cf;
    return SEM_OK;
}

// r = unmask(b - sum_j c_j b_j): the projection's residual in the continuous
// format, without an operator apply (each stored pair meets A z_j = b_j to
// the solver tolerance, far below the projection residual)
static int proj_residual(sem_ctx* c, const double* slots, const std::vector<double>& cf, const double* b, double* r)
{
    PtrList L{};
    L.nz = (int)cf.size() + 1;
    L.z[0] = b;
    L.c[0] = 1.0;
    for (int j = 0; j < (int)cf.size(); ++j) {
        L.z[j + 1] = slots + (size_t)j * 4 * c->n + 2 * c->n;
        L.c[j + 1] = -cf[j];
    }
    k_lincomb_n<<<grid_1d(2 * c->n), 256, 0, c->stream>>>(2 * c->n, L, r);
    c->stats.kernel_launches++;
    SEM_CUDA(cudaGetLastError());
    for (int q = 0; q < 2; ++q)
        SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
            return launch_unmask<decltype(nv)::value>(c->dm, false, r + q * c->n, c->stream);
        }));
    return SEM_OK;
}

// store the solved stage (z, b) in the next slot and its Gram row (d, bb
// from proj_dots with the same b)
static int proj_push(sem_ctx* c, double* slots, const double* z, const double* b, const std::vector<double>& d,
                     double bb)
{
    const int K = c->proj_k;
    const int h = c->proj_head;
    double* slot = slots + (size_t)h * 4 * c->n;
    SEM_CUDA(cudaMemcpyAsync(slot, z, sizeof(double) * 2 * c->n, cudaMemcpyDeviceToDevice, c->stream));
    SEM_CUDA(cudaMemcpyAsync(slot + 2 * c->n, b, sizeof(double) * 2 * c->n, cudaMemcpyDeviceToDevice, c->stream));
    for (int j = 0; j < c->proj_count; ++j) {
        if (j == h) continue;
        c->proj_G[(size_t)h * K + j] = c->proj_G[(size_t)j * K + h] = d[j];
    }
    c->proj_G[(size_t)h * K + h] = bb;
    c->proj_head = (h + 1) % K;
    c->proj_count = std::min(c->proj_count + 1, K);
    return SEM_OK;
}

static int schro_sdirk(sem_ctx* c, int stages, double* psi_re, double* psi_im, const double* V,
                       double T, const sem_solver_opts* o, sem_step_callback cb, void* user,
                       int* success)
{
    SEM_CHECK_CTX(c);
    if (!psi_re || !psi_im || !V || !o || !success) return fail(SEM_ERR_ARG, "null argument");
    // the reference loops while t < T with t += dt (schrodinger.hpp:219,268,
    // 376,406): a step that is not positive would never end the run
    if (!(o->dt > 0)) return fail(SEM_ERR_ARG, "dt must be positive");
    SchroRun r{};
    int s = schro_begin(c, psi_re, psi_im, V, &r);
    if (s) return s;
    double alpha;
    std::vector<std::vector<double>> arow;
    std::vector<double> bw, ew;
    if (stages == 3) {
        // schrodinger.hpp:297-301, 385, 393, 401
        const double gamma = std::cos(M_PI / 18.0) / std::sqrt(3.0) + 0.5;
        const double delta = 1.0 / 6.0 / std::pow(2 * gamma - 1, 2);
        alpha = gamma * o->dt;
        arow = {{}, {0.5 - gamma}, {2 * gamma, 1 - 4 * gamma}};
        bw = {delta, 1 - 2 * delta, delta};
    } else {
        // schrodinger.hpp:142, 228-262 (Hairer-Wanner SDIRK4, 5 stages)
        alpha = 0.25 * o->dt;
        arow = {{},
                {0.5},
                {17.0 / 50.0, -1.0 / 25.0},
                {371.0 / 1360.0, -137.0 / 2720.0, 15.0 / 544.0},
                {25.0 / 24.0, -49.0 / 48.0, 125.0 / 16.0, -85.0 / 12.0}};
        bw = {25.0 / 24.0, -49.0 / 48.0, 125.0 / 16.0, -85.0 / 12.0, 0.25};
        ew = {-3.0 / 16.0, -27.0 / 32.0, 25.0 / 32.0, 0.0, 0.25};
    }
    // stage solutions of the current and the three previous steps (ring of 4)
    const size_t zset = (size_t)stages * 2 * c->n;
    constexpr int RING = 4;
    const bool extrap = (c->guess == SEM_GUESS_EXTRAPOLATE || c->guess == SEM_GUESS_LEARNED) &&
                        c->prec == SEM_PREC_MIXED;
    // the stage history carries over from the previous driver call when it
    // continued the same kind of step (a wrong history only costs iterations:
    // every stage is still solved to the same tolerance) and starts from the
    // state that call ended with (same squared norms of both planes, bit for
    // bit: the dots have a fixed summation order)
    double sig[2] = {0.0, 0.0};
    if (extrap) {
        if ((s = dot_dev(c, r.P[r.cur], r.P[r.cur], &sig[0])) ||
            (s = dot_dev(c, r.P[r.cur] + c->n, r.P[r.cur] + c->n, &sig[1])))
            return s;
    }
    if (!extrap || c->hist_stages != stages || c->hist_dt != o->dt || sig[0] != c->hist_sig[0] ||
        sig[1] != c->hist_sig[1]) {
        c->hist_steps = 0;
        c->proj_count = c->proj_head = 0;
        c->lr_nrm2 = -1.0;
    }
    const bool proj = extrap && c->proj_k > 0;
    double* pslots = nullptr;
    if (proj && (s = proj_slots(c, &pslots))) return s;
    c->hist_stages = stages;
    c->hist_dt = o->dt;
    const long long hist0 = c->hist_steps;
    double* Zring = nullptr;
    double* Z = nullptr;
    double* b = nullptr;
    if ((s = wsget(c, "drv_Z", (extrap ? RING : 1) * zset, &Zring))) return s;
    Z = Zring;
    if ((s = wsget(c, "drv_b2", 2 * c->n, &b))) return s;
    double pnorm = 0.0;
    if (stages == 5) {
        double a1 = 0, a2 = 0;
        if ((s = dot_dev(c, r.P[0], r.P[0], &a1)) || (s = dot_dev(c, r.P[0] + c->n, r.P[0] + c->n, &a2))) return s;
        pnorm = std::sqrt(a1 + a2);  // schrodinger.hpp:214
    }
    bool ok = true;
    double t = 0.0;
    int step = 0;
    while (t < T) {  // schrodinger.hpp:219, 376
        c->stats.last_step_stages = stages;
        const long long gstep = hist0 + step;  // steps of this trajectory so far
        if (extrap) Z = Zring + (size_t)(gstep % RING) * zset;
        for (int st = 0; st < stages; ++st) {
            ZList zl{};
            zl.nz = st;
            for (int l = 0; l < st; ++l) {
                zl.z[l] = Z + (size_t)l * 2 * c->n;
                zl.c[l] = arow[st][l];
            }
            if ((s = schro_rhs(&r, o->dt, zl, b))) return s;
            double* z = Z + (size_t)st * 2 * c->n;
            // initial guess: zero as the reference (schrodinger.hpp:222,379), or
            // the projection onto the stored stage solutions (SEM_OPT_PROJECT),
            // or the stage's solution extrapolated from the previous steps:
            // linear 2 z1 - z2, or (SEM_OPT_EXTRAP_ORDER 2) quadratic
            // 3 z1 - 3 z2 + z3
            int x_zero = 1;
            auto hz = [&](long long back) {
                return Zring + (size_t)((gstep - back) % RING) * zset + (size_t)st * 2 * c->n;
            };
            std::vector<double> pd, pcf;
            double pbb = 0.0;
            bool projected = false;
            if (proj && (s = proj_dots(c, b, pslots, pd, &pbb))) return s;
            if (proj && c->proj_count > 0) {
                double ratio = 1.0;
                if ((s = proj_guess(c, pslots, pd, pbb, z, &ratio, &pcf))) return s;
                projected = true;
                c->stats.projected_guesses++;
                c->stats.last_projection_ratio = ratio;
                c->stats.projection_ratio_sum += ratio;
                x_zero = 0;
            } else if (extrap && gstep >= 1) {
                const double* z1 = hz(1);
                if (gstep >= 3 && c->extrap_order == 2) {
                    ZList q{};
                    q.nz = 3;
                    q.z[0] = z1;
                    q.c[0] = 3.0;
                    q.z[1] = hz(2);
                    q.c[1] = -3.0;
                    q.z[2] = hz(3);
                    q.c[2] = 1.0;
                    k_lincomb<<<grid_1d(2 * c->n), 256, 0, c->stream>>>(2 * c->n, q, z);
                    c->stats.kernel_launches++;
                    SEM_CUDA(cudaGetLastError());
                } else if (gstep >= 2) {
                    const double* z2 = hz(2);
                    k_axpby<<<grid_1d(2 * c->n), 256, 0, c->stream>>>(2 * c->n, 2.0, z1, -1.0, z2, z);
                    c->stats.kernel_launches++;
                    SEM_CUDA(cudaGetLastError());
                } else {
                    SEM_CUDA(cudaMemcpyAsync(z, z1, sizeof(double) * 2 * c->n, cudaMemcpyDeviceToDevice, c->stream));
                }
                x_zero = 0;
            } else {
                SEM_CUDA(cudaMemsetAsync(z, 0, sizeof(double) * 2 * c->n, c->stream));
            }
            // learned correction of the extrapolated guess, and/or a training
            // sample (the guess's residual features; its error after the solve)
            const bool rec = extrap && gstep >= 2 && !x_zero && c->ds_cap > 0;
            const bool use = extrap && gstep >= 2 && !x_zero && c->guess == SEM_GUESS_LEARNED && c->learner;
            double* zext = nullptr;
            if (rec || use) {
                double* rp = nullptr;
                if (projected) {
                    if ((s = wsget(c, "proj_r", 2 * c->n, &rp)) || (s = proj_residual(c, pslots, pcf, b, rp)))
                        return s;
                }
                if ((s = learned_guess(c, r.V, alpha, b, z, use, &zext, rp))) return s;
            }
            sem_solver_results res{};
            int sw = 1;
            if ((s = schro_stage_solve(&r, alpha, b, z, o->max_iter, o->tol, x_zero, &res, &sw)) ||
                (s = learned_collect(c)))
                return s;
            c->stats.last_stage_iters[st] = res.n_iter;
            c->stats.last_stage_sweeps[st] = sw;
            if (rec && res.success) {
                if ((s = record_sample(c, z, zext))) return s;
            }
            if (!res.success) {
                ok = false;
                break;
            }
            if (proj && (s = proj_push(c, pslots, z, b, pd, pbb))) return s;
        }
        if (!ok) {
            c->hist_steps = 0;
            c->proj_count = c->proj_head = 0;
            break;
        }
        ZList zb{};
        zb.nz = stages;
        for (int l = 0; l < stages; ++l) {
            zb.z[l] = Z + (size_t)l * 2 * c->n;
            zb.c[l] = bw[l];
        }
        SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
            return launch_update<decltype(nv)::value>(c->dm, r.P[r.cur], zb, r.P[1 - r.cur], c->stream);
        }));
        r.cur = 1 - r.cur;
        if (stages == 5) {  // embedded error estimate (schrodinger.hpp:262-263)
            double* err = nullptr;
            if ((s = wsget(c, "drv_err", 2 * c->n, &err))) return s;
            ZList ze{};
            ze.nz = 0;
            for (int l = 0; l < 5; ++l)
                if (ew[l] != 0.0) {
                    ze.z[ze.nz] = Z + (size_t)l * 2 * c->n;
                    ze.c[ze.nz++] = ew[l];
                }
            k_lincomb<<<grid_1d(2 * c->n), 256, 0, c->stream>>>(2 * c->n, ze, err);
            c->stats.kernel_launches++;
            SEM_CUDA(cudaGetLastError());
            double a1 = 0, a2 = 0;
            if ((s = dot_dev(c, err, err, &a1)) || (s = dot_dev(c, err + c->n, err + c->n, &a2))) return s;
            c->stats.last_error_estimate = std::sqrt(a1 + a2) / pnorm;
        }
        t += o->dt;
        ++step;
        c->hist_steps = hist0 + step;
        c->stats.steps_taken = step;
        if (cb) {
            if ((s = schro_publish(&r))) return s;
            if (cb(user, step, psi_re, psi_im)) break;
        }
    }
    if (extrap && ok) {
        if ((s = dot_dev(c, r.P[r.cur], r.P[r.cur], &c->hist_sig[0])) ||
            (s = dot_dev(c, r.P[r.cur] + c->n, r.P[r.cur] + c->n, &c->hist_sig[1])))
            return s;
    }
    if ((s = schro_publish(&r))) return s;
    *success = ok ? 1 : 0;
    return SEM_OK;
}

// Adaptive SDIRK4 5-stage (no counterpart in the reference, whose 5-stage
// driver computes the embedded estimate, schrodinger.hpp:262-263, but keeps
// dt fixed): a step is accepted when the estimate |sum_l e_l z_l| / |psi_0|
// is at most err_tol, and the next dt is dt * clamp(0.9 (err_tol/err)^(1/4),
// 0.2, 2) (0.2 .. 0.9 after a rejection); the last step lands on T.
extern "C" int sem_schrodinger_dirk4s5_adaptive(sem_ctx* c, double* psi_re, double* psi_im, const double* V,
                                                double T, const sem_solver_opts* o, double err_tol, double* dts,
                                                int dts_capacity, int* n_accepted, int* n_rejected,
                                                sem_step_callback cb, void* user, int* success)
{
    SEM_CHECK_CTX(c);
    if (!psi_re || !psi_im || !V || !o || !success) return fail(SEM_ERR_ARG, "null argument");
    if (!(o->dt > 0) || !(err_tol > 0) || dts_capacity < 0 || (dts_capacity > 0 && !dts))
        return fail(SEM_ERR_ARG, "bad adaptive step arguments");
    SchroRun r{};
    int s = schro_begin(c, psi_re, psi_im, V, &r);
    if (s) return s;
    // schrodinger.hpp:228-262 (Hairer-Wanner SDIRK4, 5 stages, embedded estimate)
    const std::vector<std::vector<double>> arow = {{},
                                                   {0.5},
                                                   {17.0 / 50.0, -1.0 / 25.0},
                                                   {371.0 / 1360.0, -137.0 / 2720.0, 15.0 / 544.0},
                                                   {25.0 / 24.0, -49.0 / 48.0, 125.0 / 16.0, -85.0 / 12.0}};
    const double bw[5] = {25.0 / 24.0, -49.0 / 48.0, 125.0 / 16.0, -85.0 / 12.0, 0.25};
    const double ew[5] = {-3.0 / 16.0, -27.0 / 32.0, 25.0 / 32.0, 0.0, 0.25};
    const size_t zset = (size_t)5 * 2 * c->n;
    double *Zs = nullptr, *b = nullptr, *err = nullptr;
    if ((s = wsget(c, "ad_Z", 2 * zset, &Zs)) || (s = wsget(c, "drv_b2", 2 * c->n, &b)) ||
        (s = wsget(c, "drv_err", 2 * c->n, &err)))
        return s;
    double* Z = Zs;
    double* Zp = Zs + zset;  // stage solutions of the last accepted step
    double a1 = 0, a2 = 0;
    if ((s = dot_dev(c, r.P[0], r.P[0], &a1)) || (s = dot_dev(c, r.P[0] + c->n, r.P[0] + c->n, &a2))) return s;
    const double pnorm = std::sqrt(a1 + a2);  // schrodinger.hpp:214
    const bool guess = c->guess != SEM_GUESS_ZERO && c->prec == SEM_PREC_MIXED;
    double t = 0.0, dt = o->dt, dt_prev = 0.0;
    int acc = 0, rej = 0;
    bool ok = true, have_prev = false;
    while (t < T) {
        if (T - t < dt) dt = T - t;
        if (!(dt > 1e-10 * o->dt)) {  // the controller cannot reach the tolerance
            ok = false;
            break;
        }
        const double alpha = 0.25 * dt;
        c->stats.last_step_stages = 5;
        for (int st = 0; st < 5 && ok; ++st) {
            ZList zl{};
            zl.nz = st;
            for (int l = 0; l < st; ++l) {
                zl.z[l] = Z + (size_t)l * 2 * c->n;
                zl.c[l] = arow[st][l];
            }
            if ((s = schro_rhs(&r, dt, zl, b))) return s;
            double* z = Z + (size_t)st * 2 * c->n;
            int x_zero = 1;
            if (guess && have_prev) {  // the last step's stage, scaled to this dt
                k_axpby<<<grid_1d(2 * c->n), 256, 0, c->stream>>>(2 * c->n, dt / dt_prev,
                                                                   Zp + (size_t)st * 2 * c->n, 0.0, nullptr, z);
                c->stats.kernel_launches++;
                SEM_CUDA(cudaGetLastError());
                x_zero = 0;
            } else {
                SEM_CUDA(cudaMemsetAsync(z, 0, sizeof(double) * 2 * c->n, c->stream));
            }
            // learned correction of the scaled stage of the last step, and/or
            // a training sample, as in the fixed-step drivers (the features
            // carry alpha, so one network serves every dt of the run)
            const bool rec = !x_zero && c->ds_cap > 0;
            const bool use = !x_zero && c->guess == SEM_GUESS_LEARNED && c->learner;
            double* zext = nullptr;
            if ((rec || use) && (s = learned_guess(c, r.V, alpha, b, z, use, &zext, nullptr))) return s;
            sem_solver_results res{};
            int sw = 1;
            if ((s = schro_stage_solve(&r, alpha, b, z, o->max_iter, o->tol, x_zero, &res, &sw)) ||
                (s = learned_collect(c)))
                return s;
            c->stats.last_stage_iters[st] = res.n_iter;
            c->stats.last_stage_sweeps[st] = sw;
            if (rec && res.success && (s = record_sample(c, z, zext))) return s;
            if (!res.success) ok = false;
        }
        if (!ok) break;
        ZList ze{};
        for (int l = 0; l < 5; ++l)
            if (ew[l] != 0.0) {
                ze.z[ze.nz] = Z + (size_t)l * 2 * c->n;
                ze.c[ze.nz++] = ew[l];
            }
        k_lincomb<<<grid_1d(2 * c->n), 256, 0, c->stream>>>(2 * c->n, ze, err);
        c->stats.kernel_launches++;
        SEM_CUDA(cudaGetLastError());
        if ((s = dot_dev(c, err, err, &a1)) || (s = dot_dev(c, err + c->n, err + c->n, &a2))) return s;
        const double est = std::sqrt(a1 + a2) / pnorm;
        c->stats.last_error_estimate = est;
        const double fac = est > 0 ? 0.9 * std::pow(err_tol / est, 0.25) : 2.0;
        if (est <= err_tol) {
            ZList zb{};
            zb.nz = 5;
            for (int l = 0; l < 5; ++l) {
                zb.z[l] = Z + (size_t)l * 2 * c->n;
                zb.c[l] = bw[l];
            }
            SEM_LAUNCH(dispatch_n(c->N, [&](auto nv) {
                return launch_update<decltype(nv)::value>(c->dm, r.P[r.cur], zb, r.P[1 - r.cur], c->stream);
            }));
            r.cur = 1 - r.cur;
            t += dt;
            if (acc < dts_capacity) dts[acc] = dt;
            ++acc;
            std::swap(Z, Zp);
            dt_prev = dt;
            have_prev = true;
            c->stats.steps_taken = acc;
            dt *= std::min(2.0, std::max(0.2, fac));
            if (cb) {
                if ((s = schro_publish(&r))) return s;
                if (cb(user, acc, psi_re, psi_im)) break;
            }
        } else {
            ++rej;
            dt *= std::min(0.9, std::max(0.2, fac));
        }
    }
    if ((s = schro_publish(&r))) return s;
    if (n_accepted) *n_accepted = acc;
    if (n_rejected) *n_rejected = rej;
    *success = ok ? 1 : 0;
    return SEM_OK;
}

extern "C" int sem_schrodinger_dirk4s3(sem_ctx* c, double* psi_re, double* psi_im, const double* V,
                                       double T, const sem_solver_opts* o, sem_step_callback cb,
                                       void* user, int* success)
{
    return schro_sdirk(c, 3, psi_re, psi_im, V, T, o, cb, user, success);
}

extern "C" int sem_schrodinger_dirk4s5(sem_ctx* c, double* psi_re, double* psi_im, const double* V,
                                       double T, const sem_solver_opts* o, sem_step_callback cb,
                                       void* user, int* success)
{
    return schro_sdirk(c, 5, psi_re, psi_im, V, T, o, cb, user, success);
}

extern "C" int sem_schrodinger_bdf2(sem_ctx* c, double* psi_re, double* psi_im, const double* V,
                                    double T, const sem_solver_opts* o, sem_step_callback cb,
                                    void* user, int* success)
{
    SEM_CHECK_CTX(c);
    if (!psi_re || !psi_im || !V || !o || !success) return fail(SEM_ERR_ARG, "null argument");
    // the reference loops while t < T with t += dt (schrodinger.hpp:89,107)
    if (!(o->dt > 0)) return fail(SEM_ERR_ARG, "dt must be positive");
    SchroRun r{};
    int s = schro_begin(c, psi_re, psi_im, V, &r);
    if (s) return s;
    double* PS[2] = {nullptr, nullptr};
    double* b = nullptr;
    if ((s = wsget(c, "drv_PS0", 2 * c->n, &PS[0])) || (s = wsget(c, "drv_PS1", 2 * c->n, &PS[1])) ||
        (s = wsget(c, "drv_b2", 2 * c->n, &b)))
        return s;
    double alpha = o->dt;  // schrodinger.hpp:26
    int nps = 0;
    bool ok = true;
    double t = 0.0;
    int step = 0;
    double* p = r.P[0];
    while (t < T) {  // schrodinger.hpp:89
        if (nps == 2) {
            std::swap(PS[0], PS[1]);
            nps = 1;
        }
        double* dst = PS[nps];
        // proj(p) = [gproj(re); -gproj(im)] (schrodinger.hpp:69-78)
        if ((s = apply_galerkin(c, OP_MASS, nullptr, 0.0, p, nullptr, dst, nullptr, 1.0))) return s;
        if ((s = apply_galerkin(c, OP_MASS, nullptr, 0.0, p + c->n, nullptr, dst + c->n, nullptr, -1.0))) return s;
        ++nps;
        sem_solver_results res{};
        int sw = 1;
        double* x[2] = {p, p + c->n};
        c->stats.last_step_stages = 1;
        if (nps == 1) {
            const double* bb[2] = {PS[0], PS[0] + c->n};
            if ((s = run_krylov(c, OP_RES, r.V, alpha, x, bb, o->max_iter, o->tol, 0, &res, &sw))) return s;
            alpha = (2.0 / 3.0) * o->dt;
        } else {
            k_axpby<<<grid_1d(2 * c->n), 256, 0, c->stream>>>(2 * c->n, -1.0 / 3.0, PS[0], 4.0 / 3.0, PS[1], b);
            c->stats.kernel_launches++;
            SEM_CUDA(cudaGetLastError());
            const double* bb[2] = {b, b + c->n};
            if ((s = run_krylov(c, OP_RES, r.V, alpha, x, bb, o->max_iter, o->tol, 0, &res, &sw))) return s;
        }
        c->stats.last_stage_iters[0] = res.n_iter;
        c->stats.last_stage_sweeps[0] = sw;
        if ((s = sem_unmask(c, p)) || (s = sem_unmask(c, p + c->n))) return s;
        t += o->dt;
        if (!res.success) {
            ok = false;
            break;
        }
        ++step;
        c->stats.steps_taken = step;
        if (cb) {
            if ((s = schro_publish(&r))) return s;
            if (cb(user, step, psi_re, psi_im)) break;
        }
    }
    if ((s = schro_publish(&r))) return s;
    *success = ok ? 1 : 0;
    return SEM_OK;
}
