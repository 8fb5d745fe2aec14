// Batched ensembles (device side): many independent Schroedinger instances (each its own
// mesh, degree, potential and state) advanced by BDF2 together.  No
// counterpart in the reference, whose drivers step one mesh
// (include/openmp_impl/schrodinger.hpp:22-128); each instance follows that
// driver exactly, with the stage solve of the library's mixed-precision
// MINRES (FP32 inner iterations, FP64 refinement judged on the true
// residual).
//
// Execution: one persistent launch per time step for all instances.  Blocks
// take instances from a device work queue (largest first); a block advances
// its instance by one step on its own -- projection, right-hand side, the
// complete refined MINRES solve with block barriers and block reductions,
// unmask -- so instances never wait for one another and each records its
// own convergence flag and iteration count.  The step (queue reset + kernel)
// is captured once as a CUDA graph and replayed; every per-step quantity
// (history slot, BDF coefficient) is derived on the device from the
// instance's own step counter, so the same graph serves every step.  The
// staging capacity (elements per pass of the element kernels, which sets
// the threads working on one element) is chosen per degree by a timing
// sweep at setup.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>

#include "sem_internal.h"

namespace semgb {

constexpr int BATCH_TPB = 512;
constexpr int BATCH_MIN_N = 3;  // p = 2
constexpr int BATCH_MAX_N = 9;  // p = 8
constexpr size_t BATCH_SMEM_BUDGET = 96 * 1024;

struct BatchInst {
    DevMesh m;
    double* p;         // state, 2 planes, continuous format
    double* hist[2];   // projected states [M p_re; -M p_im] (masked), 2 planes each
    double* b;         // right-hand side, 2 planes
    const double* V;   // potential
    const float* pot32;
    KrylovWork<float> w;
    double* r64;       // 2 planes
    double* Y64;       // 2 planes
    float* x32;        // 2 planes
    SolveOut* out;
    int* step;         // steps taken
    int* status;       // 0 running, 1 stopped (a stage solve failed)
    long long* iters;  // inner iterations over all steps
    int kmax;          // elements per pass of the element kernels
};

struct BatchArgs {
    const BatchInst* inst;
    const int* order;  // this launch's instances (one degree), largest first
    int n;
    int* queue;
    double dt, tol;
    int maxit;
    double inner_tol, outer_scale;
    int max_sweeps, fdm;
};

template <int N>
size_t batch_smem_n(int kmax);
template <int N>
cudaError_t batch_prepare(size_t smem, int* per_sm);
template <int N>
cudaError_t batch_launch_step(const BatchArgs& ba, int grid, size_t smem, cudaStream_t st);
template <int N>
cudaError_t batch_launch_probe(const BatchInst* inst, const int* list, int nlist, int kmax, int reps, float* sink,
                               int grid, cudaStream_t st);

}  // namespace semgb

// definitions: compiled only in the instantiation units
#ifdef SEM_BATCH_DEFINE_KERNELS
#include "sem_device.cuh"
#include "sem_solvers.cuh"

namespace semgb {

template <int N>
__device__ void bdf2_instance(const BatchInst& I, const BatchArgs& ba, unsigned char* smraw, double* red,
                              MinresScal<float>& sc, double* sweep_state, float* fdmS, float* fdmL)
{
    constexpr int NN = N * N;
    const DevMesh& m = I.m;
    const long long n = m.n;
    const int k = *I.step;
    if (*I.status) return;
    double* hnew = I.hist[k & 1];
    const double* hold = I.hist[(k + 1) & 1];
    // proj(p) (galerkin.hpp:42-57 via schrodinger.hpp:69-78): mass * p per
    // element, assembled and masked; the imaginary plane negated
    for (long long idx = threadIdx.x; idx < n; idx += blockDim.x) {
        const double ms = m.mass[idx];
        I.Y64[idx] = ms * I.p[idx];
        I.Y64[n + idx] = ms * I.p[n + idx];
    }
    __syncthreads();
    const double c0 = -1.0 / 3.0, c1 = 4.0 / 3.0;  // schrodinger.hpp:102
    for (long long idx = threadIdx.x; idx < n; idx += blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            double v = dss_value<N, double, DSS_MASK>(m, I.Y64 + c * n, ni, e, idx);
            if (c == 1) v = -1.0 * v;
            hnew[c * n + idx] = v;
            I.b[c * n + idx] = (k == 0) ? v : c0 * hold[c * n + idx] + c1 * v;
        }
    }
    __syncthreads();
    // stage solve Res(alpha) p = b from p (schrodinger.hpp:97,104), alpha = dt
    // on the first step, 2 dt / 3 after (schrodinger.hpp:98-99)
    SolveArgs a{};
    a.op = OP_RES;
    a.nc = 2;
    a.pot = I.V;
    a.alpha = (k == 0) ? ba.dt : (2.0 / 3.0) * ba.dt;
    a.b[0] = I.b;
    a.b[1] = I.b + n;
    a.x[0] = I.p;
    a.x[1] = I.p + n;
    a.maxit = ba.maxit;
    a.tol = ba.tol;
    a.x_is_zero = 0;
    a.kmax = I.kmax;
    a.rel_to_b = 0;
    a.timeout_ns = 0;
    a.sync = nullptr;  // block-local
    a.out = I.out;
    MixedArgs mx{};
    mx.inner_tol = ba.inner_tol;
    mx.max_sweeps = ba.max_sweeps;
    mx.inner_maxit = ba.maxit;
    mx.r64[0] = I.r64;
    mx.r64[1] = I.r64 + n;
    mx.Y64[0] = I.Y64;
    mx.Y64[1] = I.Y64 + n;
    mx.x32[0] = I.x32;
    mx.x32[1] = I.x32 + n;
    mx.pot32 = I.pot32;
    mx.pinv32 = nullptr;
    mx.fdm = ba.fdm;
    mx.fused = 0;
    mx.outer_scale = ba.outer_scale;
    mx.adaptive = 1;
    mixed_solve<N, OP_RES, true>(m, a, I.w, mx, 0, m.E, true, smraw, red, sc, sweep_state, fdmS, fdmL);
    // unmask(p) (schrodinger.hpp:105-106): owner copies are never written here
    for (long long idx = threadIdx.x; idx < n; idx += blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const long long src = ni_gather_src(m, node_info<N>(m, e, node % N, node / N), e, idx);
        if (src != idx) {
            I.p[idx] = I.p[src];
            I.p[n + idx] = I.p[n + src];
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *I.iters += I.out->n_iter;
        if (!I.out->success) *I.status = 1;
        *I.step = k + 1;
    }
}

// one time step of every instance in ba.order (all of degree N)
template <int N>
__global__ void __launch_bounds__(BATCH_TPB, 1) k_batch_bdf2(BatchArgs ba)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[34];
    __shared__ MinresScal<float> sc;
    __shared__ double sweep_state[3];
    __shared__ float fdmS[N * N], fdmL[N];
    __shared__ __align__(16) unsigned char ibuf[sizeof(BatchInst)];
    __shared__ int next;
    BatchInst& I = *reinterpret_cast<BatchInst*>(ibuf);
    for (;;) {
        if (threadIdx.x == 0) next = atomicAdd(ba.queue, 1);
        __syncthreads();
        const int q = next;
        if (q >= ba.n) break;
        if (threadIdx.x == 0) I = ba.inst[ba.order[q]];
        __syncthreads();
        bdf2_instance<N>(I, ba, smraw, red, sc, sweep_state, fdmS, fdmL);
        __syncthreads();
    }
}

// staging-capacity probe: every block takes instances of the probed degree
// and runs `reps` block-local FP32 Res applies with capacity kmax
template <int N>
__global__ void __launch_bounds__(BATCH_TPB, 1) k_batch_probe(const BatchInst* inst, const int* list, int nlist,
                                                               int kmax, int reps, float* sink)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ __align__(16) unsigned char ibuf[sizeof(BatchInst)];
    BatchInst& I = *reinterpret_cast<BatchInst*>(ibuf);
    float* sm = (float*)smraw;
    for (int q = blockIdx.x; q < nlist; q += gridDim.x) {
        if (threadIdx.x == 0) I = inst[list[q]];
        __syncthreads();
        const DevMesh& m = I.m;
        const Fac<float> fac = fac_of<float>(m);
        load_dmat_raw<N, float>(sm, m);
        __syncthreads();
        const long long n = m.n;
        float* Y = I.w.Y[0];
        for (int r = 0; r < reps; ++r)
            for (int e0 = 0; e0 < m.E; e0 += kmax)
                apply_range<N, float, OP_RES>(
                    sm, kmax, fac, I.pot32, 0.01f, e0, min(kmax, m.E - e0),
                    [&](int, int, int, long long flat, float* u) {
                        u[0] = I.w.L[0][flat];
                        u[1] = I.w.L[0][n + flat];
                    },
                    [&](int, int, int, long long flat, const float* o) {
                        Y[flat] = o[0];
                        Y[n + flat] = o[1];
                    });
        if (threadIdx.x == 0 && sink) sink[0] = Y[0];
        __syncthreads();
    }
}

template <int N>
size_t batch_smem_n(int kmax)
{
    return std::max(range_smem_bytes<N, double, OP_RES>(kmax), range_smem_bytes<N, float, OP_RES>(kmax));
}

// shared-memory opt-in and resident blocks per SM of the step kernel
template <int N>
cudaError_t batch_prepare(size_t smem, int* per_sm)
{
    cudaError_t e = cudaFuncSetAttribute(k_batch_bdf2<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_batch_bdf2<N>, BATCH_TPB, smem);
}

template <int N>
cudaError_t batch_launch_step(const BatchArgs& ba, int grid, size_t smem, cudaStream_t st)
{
    k_batch_bdf2<N><<<grid, BATCH_TPB, smem, st>>>(ba);
    return cudaGetLastError();
}

template <int N>
cudaError_t batch_launch_probe(const BatchInst* inst, const int* list, int nlist, int kmax, int reps, float* sink,
                               int grid, cudaStream_t st)
{
    const size_t sm = batch_smem_n<N>(kmax);
    cudaError_t e = cudaFuncSetAttribute(k_batch_probe<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    k_batch_probe<N><<<grid, BATCH_TPB, sm, st>>>(inst, list, nlist, kmax, reps, sink);
    return cudaGetLastError();
}

}  // namespace semgb

#endif  // SEM_BATCH_DEFINE_KERNELS

#define SEM_BATCH_INSTANTIATE(NV)                                                                        \
    namespace semgb {                                                                                    \
    template size_t batch_smem_n<NV>(int);                                                               \
    template cudaError_t batch_prepare<NV>(size_t, int*);                                                \
    template cudaError_t batch_launch_step<NV>(const BatchArgs&, int, size_t, cudaStream_t);             \
    template cudaError_t batch_launch_probe<NV>(const BatchInst*, const int*, int, int, int, float*, int, \
                                                cudaStream_t);                                           \
    }
