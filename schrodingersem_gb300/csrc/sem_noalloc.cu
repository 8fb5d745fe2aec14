// sem_apply_schro_res_noalloc: the Schroedinger Res operator for callers
// that must not allocate device memory.
//
// The ordinary sem_apply_schro_res keeps its element-local intermediate (the
// unassembled operator output, 2*E*N*N doubles) in a workspace the library
// allocates with cudaMalloc on first use.  Some callers cannot let a library
// allocate: code whose device memory is owned and budgeted by a host
// framework or pool allocator, and latency-critical loops in which the
// implicit device synchronisation of cudaMalloc/cudaFree is not acceptable.
// This variant keeps that intermediate in a fixed, statically sized device
// array instead, so the call itself allocates nothing; the caller still
// passes the (device) inputs and outputs.
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <type_traits>

#include "sem_gb300.h"
#include "sem_internal.h"

using namespace semgb;

namespace {

// Capacity of the static scratch: 2*E*N*N must not exceed this many doubles
// (8 MiB; e.g. 4,096 elements at p = 8 need 663,552).  Every GPU that loads
// the library holds this array until the process exits.
constexpr long long kNoAllocScratchValues = 1LL << 20;

__device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchValues];

// Device address of g_noalloc_scratch per device, filled on the first call
// made on that device.  In host code the symbol g_noalloc_scratch is only a
// host-side stand-in: its address must come from cudaGetSymbolAddress with
// that device current.  The entry point runs only with the context's own
// device current (it rejects other calls), so the lookup is for that device.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {};

int scratch_for_device(int dev, double** out)
{
    if (dev < 0 || dev >= kMaxDevices) return ctx_fail(SEM_ERR_UNSUPPORTED, "device ordinal above 63");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            std::string msg = std::string("cudaGetSymbolAddress(noalloc scratch): ") + cudaGetErrorString(e);
            return ctx_fail(SEM_ERR_CUDA, msg.c_str());
        }
        g_scratch_ptr[dev] = (double*)p;
    }
    *out = g_scratch_ptr[dev];
    return SEM_OK;
}

template <class F>
cudaError_t dispatch_n_local(int N, F&& f)
{
    switch (N) {
#define SEM_CASE(NV) \
    case NV: return f(std::integral_constant<int, NV>{});
        SEM_FOR_EACH_N(SEM_CASE)
#undef SEM_CASE
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

extern "C" int sem_apply_schro_res_noalloc(sem_ctx* c, const double* V, double alpha, const double* qr,
                                           const double* qi, double* yr, double* yi)
{
    if (!c) return ctx_fail(SEM_ERR_ARG, "null ctx");
    if (!V || !qr || !qi || !yr || !yi) return ctx_fail(SEM_ERR_ARG, "null field");
    const DevMesh& m = ctx_mesh(c);
    if (2 * m.n > kNoAllocScratchValues) {
        std::string msg = "sem_apply_schro_res_noalloc: the mesh needs 2*E*N*N = " + std::to_string(2 * m.n) +
                          " scratch values, above the static capacity of " +
                          std::to_string(kNoAllocScratchValues) + "; use sem_apply_schro_res";
        return ctx_fail(SEM_ERR_UNSUPPORTED, msg.c_str());
    }
    // the context's stream and the scratch belong to the context's device
    int cur = -1;
    cudaError_t ge = cudaGetDevice(&cur);
    if (ge != cudaSuccess) return ctx_fail(SEM_ERR_CUDA, cudaGetErrorString(ge));
    if (cur != ctx_device(c))
        return ctx_fail(SEM_ERR_ARG, "sem_apply_schro_res_noalloc: make the context's device current first");
    double* Y = nullptr;
    int s = scratch_for_device(cur, &Y);
    if (s) return s;
    double* Y1 = Y + m.n;
    cudaStream_t st = ctx_stream(c);
    // the element kernel writes every scratch entry before the assembly reads
    // it, so nothing left by an earlier call needs clearing
    cudaError_t e = dispatch_n_local(m.N, [&](auto nv) {
        return launch_apply<decltype(nv)::value>(m, OP_RES, false, V, alpha, qr, qi, Y, Y1, true, st);
    });
    if (e == cudaSuccess)
        e = dispatch_n_local(m.N, [&](auto nv) {
            return launch_dss<decltype(nv)::value>(m, false, DSS_MASK, 1.0, Y, yr, st);
        });
    if (e == cudaSuccess)
        e = dispatch_n_local(m.N, [&](auto nv) {
            return launch_dss<decltype(nv)::value>(m, false, DSS_MASK, 1.0, Y1, yi, st);
        });
    if (e != cudaSuccess) {
        std::string msg = std::string("launch: ") + cudaGetErrorString(e);
        return ctx_fail(SEM_ERR_CUDA, msg.c_str());
    }
    ctx_count_launches(c, 3);
    ctx_count_fp64_apply(c);
    return SEM_OK;
}
