// Batched ensembles: many independent Schroedinger instances (each its own
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
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <type_traits>
#include <vector>

#include "sem_gb300.h"
#include "sem_internal.h"

#include "sem_batch.cuh"  // declarations; kernels instantiated in sem_batch_inst_*.cu

using namespace semgb;

namespace {
template <class F>
cudaError_t dispatch_batch_n(int N, F&& f)
{
    switch (N) {
        case 3: return f(std::integral_constant<int, 3>{});
        case 4: return f(std::integral_constant<int, 4>{});
        case 5: return f(std::integral_constant<int, 5>{});
        case 6: return f(std::integral_constant<int, 6>{});
        case 7: return f(std::integral_constant<int, 7>{});
        case 8: return f(std::integral_constant<int, 8>{});
        case 9: return f(std::integral_constant<int, 9>{});
        default: return cudaErrorInvalidValue;
    }
}
}  // namespace

// instances of one degree: their order (largest first), queue and launch shape
struct BatchGroup {
    int N = 0;
    std::vector<int> members;
    int* d_order = nullptr;
    int* d_queue = nullptr;
    int grid = 0;
    size_t smem = 0;
    cudaStream_t fork = nullptr;
    cudaEvent_t done = nullptr;
};

struct sem_batch {
    std::vector<sem_ctx*> ctx;
    std::vector<int> N;
    std::vector<long long> nloc;
    std::vector<BatchGroup> groups;
    std::vector<void*> owned;
    BatchInst* d_inst = nullptr;
    std::vector<BatchInst> h_inst;
    int* d_step = nullptr;
    int* d_status = nullptr;
    long long* d_iters = nullptr;
    cudaStream_t stream = nullptr;
    int sms = 0;
    // options
    double inner_tol = 1e-4, outer_scale = 1.0;
    int max_refine = 50, precond = SEM_PRECOND_FDM;
    sem_batch_stats stats{};
    cudaGraphExec_t graph = nullptr;
    BatchArgs graph_args{};
    cudaEvent_t fork_ev = nullptr;
};

static int bfail(int code, const std::string& msg) { return ctx_fail(code, msg.c_str()); }

#define BCUDA(call)                                                                                            \
    do {                                                                                                       \
        cudaError_t e_ = (call);                                                                               \
        if (e_ != cudaSuccess) return bfail(SEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

static int balloc(sem_batch* b, void** p, size_t bytes)
{
    cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) return bfail(SEM_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    b->owned.push_back(*p);
    return SEM_OK;
}

extern "C" int sem_batch_destroy(sem_batch* b)
{
    if (!b) return SEM_OK;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (BatchGroup& g : b->groups) {
        if (g.fork) cudaStreamDestroy(g.fork);
        if (g.done) cudaEventDestroy(g.done);
    }
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    for (void* p : b->owned) cudaFree(p);
    for (sem_ctx* c : b->ctx) sem_ctx_destroy(c);
    delete b;
    return SEM_OK;
}

// Staging capacity per degree: time block-local FP32 Res applies over the
// group's largest instances for kmax = 1, 2, 4, ... (as far as the element
// count and the shared-memory budget allow) and keep the fastest.
static int tune_group(sem_batch* b, BatchGroup& g, int* kmax_out)
{
    const int N = g.N;
    std::vector<int> list(g.members.begin(), g.members.begin() + std::min<size_t>(g.members.size(), 64));
    long long emax = 0;
    for (int i : list) emax = std::max<long long>(emax, b->nloc[i] / (N * N));
    int* dl = nullptr;
    float* sink = nullptr;
    int s = 0;
    if ((s = balloc(b, (void**)&dl, sizeof(int) * list.size())) || (s = balloc(b, (void**)&sink, sizeof(float))))
        return s;
    BCUDA(cudaMemcpy(dl, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice));
    cudaEvent_t e0, e1;
    BCUDA(cudaEventCreate(&e0));
    BCUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_k = 1;
    const int grid = std::min<int>((int)list.size(), b->sms);
    for (int kmax = 1; kmax <= 256; kmax *= 2) {
        if (kmax > 1 && kmax / 2 >= emax) break;
        size_t sm = 0;
        dispatch_batch_n(N, [&](auto nv) {
            sm = batch_smem_n<decltype(nv)::value>(kmax);
            return cudaSuccess;
        });
        if (sm > BATCH_SMEM_BUDGET) break;
        auto launch = [&]() {
            return dispatch_batch_n(N, [&](auto nv) {
                return batch_launch_probe<decltype(nv)::value>(b->d_inst, dl, (int)list.size(), kmax, 8, sink, grid,
                                                               b->stream);
            });
        };
        BCUDA(launch());  // warm-up
        BCUDA(cudaEventRecord(e0, b->stream));
        BCUDA(launch());
        BCUDA(cudaEventRecord(e1, b->stream));
        BCUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        BCUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            best_k = kmax;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *kmax_out = best_k;
    return SEM_OK;
}

extern "C" int sem_batch_create(sem_batch** out, int n_inst, const int* p, const int* n_nodes,
                                const double* const* coords, const int* n_elements, const int* const* elements,
                                unsigned flags)
{
    if (!out || n_inst <= 0 || !p || !n_nodes || !coords || !n_elements || !elements)
        return bfail(SEM_ERR_ARG, "bad batch arguments");
    *out = nullptr;
    for (int i = 0; i < n_inst; ++i)
        if (p[i] + 1 < BATCH_MIN_N || p[i] + 1 > BATCH_MAX_N)
            return bfail(SEM_ERR_UNSUPPORTED, "batched instances support p = 2..8");
    sem_batch* b = new sem_batch();
    int s = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    for (int i = 0; i < n_inst; ++i) {
        sem_ctx* c = nullptr;
        if ((s = sem_ctx_create(&c, p[i], n_nodes[i], coords[i], n_elements[i], elements[i], flags))) {
            sem_batch_destroy(b);
            return s;
        }
        b->ctx.push_back(c);
        b->N.push_back(p[i] + 1);
        b->nloc.push_back((long long)n_elements[i] * (p[i] + 1) * (p[i] + 1));
    }
    const int n = n_inst;
    // one pool per precision for all instances' vectors
    long long tot = 0;
    for (long long v : b->nloc) tot += v;
    double* pool64 = nullptr;
    float* pool32 = nullptr;
    double* vpool = nullptr;
    SolveOut* outs = nullptr;
    const long long per64 = 12, per32 = 25;  // values per local node
    if ((s = balloc(b, (void**)&pool64, sizeof(double) * per64 * tot)) ||
        (s = balloc(b, (void**)&pool32, sizeof(float) * per32 * tot)) ||
        (s = balloc(b, (void**)&vpool, sizeof(double) * tot)) ||
        (s = balloc(b, (void**)&b->d_step, sizeof(int) * n)) ||
        (s = balloc(b, (void**)&b->d_status, sizeof(int) * n)) ||
        (s = balloc(b, (void**)&b->d_iters, sizeof(long long) * n)) ||
        (s = balloc(b, (void**)&b->d_inst, sizeof(BatchInst) * n)) ||
        (s = balloc(b, (void**)&outs, sizeof(SolveOut) * n))) {
        sem_batch_destroy(b);
        return s;
    }
    if (cudaMemset(pool32, 0, sizeof(float) * per32 * tot) != cudaSuccess ||
        cudaMemset(pool64, 0, sizeof(double) * per64 * tot) != cudaSuccess) {
        sem_batch_destroy(b);
        return bfail(SEM_ERR_CUDA, "cudaMemset of the batch pools");
    }
    b->h_inst.resize(n);
    long long o64 = 0, o32 = 0, ov = 0;
    for (int i = 0; i < n; ++i) {
        const long long v = b->nloc[i];
        BatchInst& I = b->h_inst[i];
        std::memset(&I, 0, sizeof(I));
        I.m = ctx_mesh(b->ctx[i]);
        auto t64 = [&](long long cnt) {
            double* q = pool64 + o64;
            o64 += cnt;
            return q;
        };
        auto t32 = [&](long long cnt) {
            float* q = pool32 + o32;
            o32 += cnt;
            return q;
        };
        I.p = t64(2 * v);
        I.hist[0] = t64(2 * v);
        I.hist[1] = t64(2 * v);
        I.b = t64(2 * v);
        I.r64 = t64(2 * v);
        I.Y64 = t64(2 * v);
        for (int q = 0; q < 3; ++q) I.w.L[q] = t32(2 * v);
        for (int q = 0; q < 3; ++q) I.w.W[q] = t32(2 * v);
        for (int q = 0; q < 2; ++q) I.w.Y[q] = t32(2 * v);
        for (int q = 0; q < 2; ++q) I.w.Z[q] = t32(2 * v);
        I.w.Y3 = t32(2 * v);
        I.x32 = t32(2 * v);
        I.pot32 = t32(v);
        I.V = vpool + ov;
        ov += v;
        I.out = outs + i;
        I.step = b->d_step + i;
        I.status = b->d_status + i;
        I.iters = b->d_iters + i;
        I.kmax = 1;
    }
    cudaError_t e = cudaMemcpy(b->d_inst, b->h_inst.data(), sizeof(BatchInst) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        sem_batch_destroy(b);
        return bfail(SEM_ERR_CUDA, cudaGetErrorString(e));
    }
    // degree groups, largest instances first
    for (int N = BATCH_MIN_N; N <= BATCH_MAX_N; ++N) {
        BatchGroup g;
        g.N = N;
        for (int i = 0; i < n; ++i)
            if (b->N[i] == N) g.members.push_back(i);
        if (g.members.empty()) continue;
        std::stable_sort(g.members.begin(), g.members.end(), [&](int x, int y) { return b->nloc[x] > b->nloc[y]; });
        b->groups.push_back(std::move(g));
    }
    for (BatchGroup& g : b->groups) {
        int kmax = 1;
        if ((s = tune_group(b, g, &kmax))) {
            sem_batch_destroy(b);
            return s;
        }
        b->stats.kmax_of_p[g.N - 1] = kmax;
        for (int i : g.members) b->h_inst[i].kmax = kmax;
        int per_sm = 0;
        dispatch_batch_n(g.N, [&](auto nv) {
            g.smem = batch_smem_n<decltype(nv)::value>(kmax);
            return cudaSuccess;
        });
        e = dispatch_batch_n(g.N, [&](auto nv) { return batch_prepare<decltype(nv)::value>(g.smem, &per_sm); });
        if (e != cudaSuccess || per_sm < 1) {
            sem_batch_destroy(b);
            return bfail(SEM_ERR_CUDA, "batched step kernel does not fit");
        }
        g.grid = std::min<int>((int)g.members.size(), b->sms * per_sm);
        if ((s = balloc(b, (void**)&g.d_order, sizeof(int) * g.members.size())) ||
            (s = balloc(b, (void**)&g.d_queue, sizeof(int)))) {
            sem_batch_destroy(b);
            return s;
        }
        e = cudaMemcpy(g.d_order, g.members.data(), sizeof(int) * g.members.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g.fork, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            sem_batch_destroy(b);
            return bfail(SEM_ERR_CUDA, cudaGetErrorString(e));
        }
    }
    e = cudaMemcpy(b->d_inst, b->h_inst.data(), sizeof(BatchInst) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        sem_batch_destroy(b);
        return bfail(SEM_ERR_CUDA, cudaGetErrorString(e));
    }
    *out = b;
    return SEM_OK;
}

extern "C" int sem_batch_set_stream(sem_batch* b, void* stream)
{
    if (!b) return bfail(SEM_ERR_ARG, "null batch");
    b->stream = (cudaStream_t)stream;
    return SEM_OK;
}

extern "C" int sem_batch_set_option(sem_batch* b, int option, double v)
{
    if (!b) return bfail(SEM_ERR_ARG, "null batch");
    switch (option) {
        case SEM_OPT_INNER_TOL:
            if (!(v > 0 && v < 1)) return bfail(SEM_ERR_ARG, "inner tolerance must be in (0,1)");
            b->inner_tol = v;
            break;
        case SEM_OPT_MAX_REFINE:
            if (v < 1) return bfail(SEM_ERR_ARG, "max refine must be >= 1");
            b->max_refine = (int)v;
            break;
        case SEM_OPT_PRECOND:
            if (v != SEM_PRECOND_NONE && v != SEM_PRECOND_FDM)
                return bfail(SEM_ERR_ARG, "batched solves take SEM_PRECOND_NONE or SEM_PRECOND_FDM");
            b->precond = (int)v;
            break;
        case SEM_OPT_REFINE_TOL_SCALE:
            if (!(v > 0 && v <= 1)) return bfail(SEM_ERR_ARG, "refinement tolerance scale must be in (0,1]");
            b->outer_scale = v;
            break;
        case SEM_OPT_SOLVE_PRECISION:
            if (v != SEM_PREC_MIXED) return bfail(SEM_ERR_UNSUPPORTED, "batched solves are mixed precision");
            break;
        default: return bfail(SEM_ERR_ARG, "option not supported by batches");
    }
    return SEM_OK;
}

extern "C" int sem_batch_get_info(const sem_batch* b, int inst, sem_mesh_info* info)
{
    if (!b || inst < 0 || inst >= (int)b->ctx.size()) return bfail(SEM_ERR_ARG, "bad instance");
    return sem_ctx_get_info(b->ctx[inst], info);
}

extern "C" int sem_batch_get_stats(const sem_batch* b, sem_batch_stats* st)
{
    if (!b || !st) return bfail(SEM_ERR_ARG, "null argument");
    *st = b->stats;
    return SEM_OK;
}

extern "C" int sem_batch_get_instance(const sem_batch* b, int inst, int* steps, int* stopped, long long* iterations)
{
    if (!b || inst < 0 || inst >= (int)b->ctx.size()) return bfail(SEM_ERR_ARG, "bad instance");
    if (steps) BCUDA(cudaMemcpy(steps, b->d_step + inst, sizeof(int), cudaMemcpyDeviceToHost));
    if (stopped) BCUDA(cudaMemcpy(stopped, b->d_status + inst, sizeof(int), cudaMemcpyDeviceToHost));
    if (iterations) BCUDA(cudaMemcpy(iterations, b->d_iters + inst, sizeof(long long), cudaMemcpyDeviceToHost));
    return SEM_OK;
}

static bool dev_ptr(const void* p)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

namespace {
__global__ void k_to_f32_b(long long n, const double* __restrict__ a, float* __restrict__ b)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}
}  // namespace

// capture one time step: per degree group, reset its queue and launch its
// persistent kernel on a forked stream; the groups run side by side
static int capture_step(sem_batch* b, const BatchArgs& base)
{
    cudaStream_t cs = nullptr;
    BCUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaEventRecord(b->fork_ev, cs);
        for (BatchGroup& gr : b->groups) {
            cudaStreamWaitEvent(gr.fork, b->fork_ev, 0);
            BatchArgs ba = base;
            ba.order = gr.d_order;
            ba.n = (int)gr.members.size();
            ba.queue = gr.d_queue;
            cudaMemsetAsync(gr.d_queue, 0, sizeof(int), gr.fork);
            dispatch_batch_n(gr.N, [&](auto nv) {
                return batch_launch_step<decltype(nv)::value>(ba, gr.grid, gr.smem, gr.fork);
            });
            cudaEventRecord(gr.done, gr.fork);
            cudaStreamWaitEvent(cs, gr.done, 0);
        }
        e = cudaStreamEndCapture(cs, &g);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return bfail(SEM_ERR_CUDA, std::string("step graph: ") + cudaGetErrorString(e));
    b->stats.graphs_built++;
    return SEM_OK;
}

extern "C" int sem_batch_schrodinger_bdf2(sem_batch* b, double* const* psi_re, double* const* psi_im,
                                          const double* const* V, double T, const sem_solver_opts* opts,
                                          int* success)
{
    if (!b || !psi_re || !psi_im || !V || !opts || !success) return bfail(SEM_ERR_ARG, "null argument");
    if (!(opts->dt > 0)) return bfail(SEM_ERR_ARG, "dt must be positive");
    const int n = (int)b->ctx.size();
    // inputs: state (unmasked, as the reference's wrappers hold it) and potential
    for (int i = 0; i < n; ++i) {
        const BatchInst& I = b->h_inst[i];
        const long long v = b->nloc[i];
        if (!psi_re[i] || !psi_im[i] || !V[i]) return bfail(SEM_ERR_ARG, "null instance field");
        const cudaMemcpyKind kr = dev_ptr(psi_re[i]) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        const cudaMemcpyKind kv = dev_ptr(V[i]) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        BCUDA(cudaMemcpyAsync(I.p, psi_re[i], sizeof(double) * v, kr, b->stream));
        BCUDA(cudaMemcpyAsync(I.p + v, psi_im[i], sizeof(double) * v, kr, b->stream));
        BCUDA(cudaMemcpyAsync((void*)I.V, V[i], sizeof(double) * v, kv, b->stream));
        k_to_f32_b<<<(int)std::min<long long>((v + 255) / 256, 1024), 256, 0, b->stream>>>(v, I.V, (float*)I.pot32);
        BCUDA(cudaGetLastError());
    }
    BCUDA(cudaMemsetAsync(b->d_step, 0, sizeof(int) * n, b->stream));
    BCUDA(cudaMemsetAsync(b->d_status, 0, sizeof(int) * n, b->stream));
    BCUDA(cudaMemsetAsync(b->d_iters, 0, sizeof(long long) * n, b->stream));
    BatchArgs ba{};
    ba.inst = b->d_inst;
    ba.dt = opts->dt;
    ba.tol = opts->tol;
    ba.maxit = opts->max_iter;
    ba.inner_tol = b->inner_tol;
    ba.outer_scale = b->outer_scale;
    ba.max_sweeps = b->max_refine;
    ba.fdm = b->precond == SEM_PRECOND_FDM ? 1 : 0;
    if (b->graph && std::memcmp(&ba, &b->graph_args, sizeof(BatchArgs)) != 0) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    if (!b->graph) {
        const int s = capture_step(b, ba);
        if (s) return s;
        b->graph_args = ba;
    }
    // the reference's time loop: while (t < T) { ...; t += dt } (schrodinger.hpp:89,107)
    int steps = 0;
    for (double t = 0.0; t < T; t += opts->dt) ++steps;
    cudaEvent_t e0, e1;
    BCUDA(cudaEventCreate(&e0));
    BCUDA(cudaEventCreate(&e1));
    BCUDA(cudaEventRecord(e0, b->stream));
    for (int k = 0; k < steps; ++k) BCUDA(cudaGraphLaunch(b->graph, b->stream));
    BCUDA(cudaEventRecord(e1, b->stream));
    BCUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->stats.steps += steps;
    b->stats.graph_launches += steps;
    b->stats.kernel_ms += ms;
    // outputs and flags
    std::vector<int> st(n);
    std::vector<long long> it(n);
    BCUDA(cudaMemcpy(st.data(), b->d_status, sizeof(int) * n, cudaMemcpyDeviceToHost));
    BCUDA(cudaMemcpy(it.data(), b->d_iters, sizeof(long long) * n, cudaMemcpyDeviceToHost));
    long long tot_it = 0;
    for (int i = 0; i < n; ++i) {
        const BatchInst& I = b->h_inst[i];
        const long long v = b->nloc[i];
        const cudaMemcpyKind kr = dev_ptr(psi_re[i]) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        BCUDA(cudaMemcpyAsync(psi_re[i], I.p, sizeof(double) * v, kr, b->stream));
        BCUDA(cudaMemcpyAsync(psi_im[i], I.p + v, sizeof(double) * v, kr, b->stream));
        success[i] = st[i] ? 0 : 1;
        tot_it += it[i];
    }
    BCUDA(cudaStreamSynchronize(b->stream));
    b->stats.krylov_iterations += tot_it;
    b->stats.instance_steps += (long long)steps * n;
    return SEM_OK;
}
