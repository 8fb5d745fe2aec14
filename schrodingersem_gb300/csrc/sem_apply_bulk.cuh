// Pipelined element operator for the standalone applies.
//
// A persistent grid walks the mesh in batches of K elements (K N^2 nodes,
// contiguous in every field).  For each batch one thread issues a 1-D bulk
// copy (cp.async.bulk, completion counted on an mbarrier) of every array the
// operator reads -- the inputs, the premultiplied factors, the potential --
// into one of S shared-memory stages, so S batches of loads are in flight
// per block while the block computes on the oldest.  Inputs in the masked
// format are then patched at the ring copies that are not the owner (their
// value is read from the owner copy, the reference's unmask), the two
// contraction phases run from shared memory, and the element-local result
// is stored with coalesced stores.  A batch shorter than K (the mesh tail)
// is loaded with plain loads instead: bulk copies need 16-byte sizes.
//
// Every wait on an mbarrier is bounded (globaltimer); on expiry the block
// records an error in DevMesh::dev_err, waits (bounded) for its own copies
// in flight and returns.
#pragma once
#include <cstdint>
#include <cstring>
#include <mutex>

#include "sem_device.cuh"

namespace semgb {

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// arrive (count 1) and add `bytes` to the transaction count of this phase
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// wait for phase `parity` of the barrier to complete, at most timeout_ns
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long timeout_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned int it = 1;; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 15u) == 0 && (long long)(global_ns() - t0) > timeout_ns) return false;
    }
}

// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// order this thread's generic shared-memory accesses before later
// async-proxy (bulk copy) writes to the same memory
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// shared -> global bulk copy (bulk-group completion); 16-byte aligned, size a
// multiple of 16
__device__ __forceinline__ void bulk_store(void* dst, const void* src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the shared-memory sources of all committed bulk stores have been read
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// all committed bulk stores have completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// arrays staged per batch: inputs (NC), then g11 g12 g22 (not for the mass
// operator), mass (not for Laplace), potential (Helmholtz, Res, f)
template <int OP>
__host__ __device__ constexpr int bulk_arrays()
{
    return op_nc<OP>() + (OP == OP_MASS ? 0 : 3) + (OP == OP_LAPLACE ? 0 : 1) +
           ((OP == OP_HELM || OP == OP_RES || OP == OP_F) ? 1 : 0);
}
// with the geometric factors computed on the fly (GEO, Res only): the two
// inputs and the potential per node, plus 8 corner differences per element
template <int OP, bool GEO>
__host__ __device__ constexpr int bulk_arrays_g()
{
    return GEO ? op_nc<OP>() + 1 : bulk_arrays<OP>();
}
constexpr int GEO_PER_EL = 8;  // x1-x0, x2-x3, x3-x0, x2-x1, and the same for y

// threads per block: one per element line and component
template <typename T, int OP>
__host__ __device__ constexpr int bulk_tpb()
{
    return (sizeof(T) == 4 ? 128 : 64) * op_nc<OP>();
}

// threads of the kernel: with MG (Res) one thread per line works on both
// components
template <typename T, int OP, bool MG>
__host__ __device__ constexpr int bulk_tpb_k()
{
    return MG ? bulk_tpb<T, OP>() / op_nc<OP>() : bulk_tpb<T, OP>();
}

constexpr int BULK_STAGES = 2;  // one batch in flight while one computes (3 measured slower)
constexpr size_t BULK_SMEM_TARGET = 72 * 1024;  // three blocks per SM

// elements per batch: one line thread per element column (K N <= threads),
// BULK_STAGES stages of every staged array plus two work planes per
// component within BULK_SMEM_TARGET; a multiple of 4 (FP32) or 2 (FP64) so that a batch of
// any field is a multiple of 16 bytes
template <typename T, int OP>
__host__ __device__ constexpr int bulk_k(int N)
{
    const int q = sizeof(T) == 4 ? 4 : 2;
    const int by_lines = bulk_tpb<T, OP>() / op_nc<OP>() / N;
    const int per_node = (BULK_STAGES * bulk_arrays<OP>() + 2 * op_nc<OP>()) * (int)sizeof(T);
    const int by_smem = (int)(BULK_SMEM_TARGET / (size_t)(per_node * N * N));
    const int k = (by_lines < by_smem ? by_lines : by_smem) / q * q;
    return k < q ? q : k;
}

template <int N, typename T, int OP, bool GEO = false>
__host__ __device__ constexpr size_t bulk_smem_bytes()
{
    return 128 + (size_t)(BULK_STAGES * bulk_arrays_g<OP, GEO>() + 2 * op_nc<OP>()) * bulk_k<T, OP>(N) * N * N *
                     sizeof(T) +
           (GEO ? (size_t)BULK_STAGES * bulk_k<T, OP>(N) * GEO_PER_EL * sizeof(float) : 0);
}

// 0.25 (1 - z_i), 0.25 (1 + z_i) and w_i of the LGL nodes, and the metric
// convention, passed by value (constant-bank operands of the on-the-fly
// geometric factors)
template <int N>
struct GeoTab {
    float lo[N], hi[N], w[N];
    int corrected;
};

// premultiplied factors of node (i, j) from the element's corner differences
// g (include/Quad.hpp:39-54 as the library's setup evaluates them, in FP32):
// X_xi, Y_xi at eta_j, X_eta, Y_eta at xi_i, J, and w_i w_j {A, B, C, J}.
// The thread's own line coordinate (lo, hi, w of its l) comes in registers
// and the unrolled one from the table, so no index into the table is a
// runtime value.
struct GeoLine {
    float lo, hi, w;
};
template <int N>
__device__ __forceinline__ GeoLine geo_line(const GeoTab<N>& gt, int l)
{
    GeoLine r{0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < N; ++k)
        if (k == l) r = GeoLine{gt.lo[k], gt.hi[k], gt.w[k]};
    return r;
}
// node (i, l): i unrolled, j = l the thread's column line
template <int N>
__device__ __forceinline__ void geo_factors_col(const GeoTab<N>& gt, const float* g, int i, const GeoLine& lj,
                                                float& g11, float& g12, float& g22)
{
    const float xxi = lj.lo * g[0] + lj.hi * g[1], yxi = lj.lo * g[4] + lj.hi * g[5];
    const float xet = gt.lo[i] * g[2] + gt.hi[i] * g[3], yet = gt.lo[i] * g[6] + gt.hi[i] * g[7];
    const float yx = gt.corrected ? yxi : gt.lo[i] * g[4] + gt.hi[i] * g[5];
    const float J = xxi * yet - xet * yxi;
    const float r = (gt.w[i] * lj.w) / J;
    g11 = (yet * yet + xet * xet) * r;
    g12 = (yet * yxi + xet * xxi) * r;
    g22 = (yx * yx + xxi * xxi) * r;
}
// w_i w_j J of node (l, j): i = l the thread's row line, j unrolled
template <int N>
__device__ __forceinline__ float geo_mass_row(const GeoTab<N>& gt, const float* g, const GeoLine& li, int j)
{
    const float xxi = gt.lo[j] * g[0] + gt.hi[j] * g[1], yxi = gt.lo[j] * g[4] + gt.hi[j] * g[5];
    const float xet = li.lo * g[2] + li.hi * g[3], yet = li.lo * g[6] + li.hi * g[7];
    return (li.w * gt.w[j]) * (xxi * yet - xet * yxi);
}

// D(i,k) at [i*N+k], passed by value: the kernel reads it from the constant
// bank as an operand of its FMAs
template <int N, typename T>
struct DMat {
    T d[N * N];
};

// D(i,k) duplicated into both lanes of a packed FP32 pair, for the paired
// FMA of the two Res components (each lane an IEEE FP32 FMA: same bits as
// two scalar FMAs)
template <int N>
struct DMat2 {
    unsigned long long d[N * N];
};
__device__ __forceinline__ unsigned long long f2pack(float a, float b)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2unpack(unsigned long long v, float& a, float& b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2fma(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// Line contraction of both Res components: oa[o] = ca[o] + sum_k M(o,k) a[k]
// (and b) with M = D (TR false) or D^T (TR true), k ascending; paired FP32
// FMAs when F2 (measured faster for N <= 11, slower above), else scalar.
template <int N, bool TR, bool F2>
__device__ __forceinline__ void contract2(const DMat<N, float>& D, const DMat2<N>& D2, const float* a,
                                          const float* b, float* oa, float* ob)
{
    if constexpr (F2) {
        unsigned long long v[N], acc[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
            v[i] = f2pack(a[i], b[i]);
            acc[i] = f2pack(oa[i], ob[i]);
        }
#pragma unroll
        for (int k = 0; k < N; ++k)
#pragma unroll
            for (int o = 0; o < N; ++o) acc[o] = f2fma(D2.d[TR ? k * N + o : o * N + k], v[k], acc[o]);
#pragma unroll
        for (int o = 0; o < N; ++o) f2unpack(acc[o], oa[o], ob[o]);
    } else {
#pragma unroll
        for (int k = 0; k < N; ++k)
#pragma unroll
            for (int o = 0; o < N; ++o) {
                const float dk = D.d[TR ? k * N + o : o * N + k];
                oa[o] = fma(dk, a[k], oa[o]);
                ob[o] = fma(dk, b[k], ob[o]);
            }
    }
}
__host__ __device__ constexpr bool bulk_f2(int N) { return N <= 11; }

// One batch = K elements.  After the stage of a batch has arrived (and, for
// masked inputs, its non-owner ring copies are patched), thread
// t = le*N + l works on line l of element le (with MG, Res only, on both
// components, which shares the factor loads and fuses P3 with P4; without
// MG, threads t and t + TPB/2 take the two components):
//   P1  column l: ur(:,l) = D u(:,l) (kept in registers);
//       row l:    us(l,:) = u(l,:) D^T          -> W1
//   P2  column l: f1 = g11 ur - g12 us, f2 = g22 us - g12 ur; f2 -> W1,
//       lap1(:,l) = D^T f1(:,l)                 -> W2
//   P3  row l:    lap(l,:) = lap1(l,:) + f2(l,:) D, then the mass/potential
//       epilogue of the operator                -> W2
// and W2 is written out with one bulk store per component.  Every
// accumulation runs over k in ascending order as in apply_chunk (the
// one-pass kernel), so both kernels give the same bits.
template <int N, typename T, int OP, bool GATHER, bool MG, bool GEO = false>
__global__ void __launch_bounds__(bulk_tpb_k<T, OP, MG>())
    k_apply_bulk(DevMesh m, DMat<N, T> D, DMat2<N> D2, const T* __restrict__ pot, T alpha, const T* __restrict__ in0,
                 const T* __restrict__ in1, T* __restrict__ y0, T* __restrict__ y1, int store_bulk, int pair_asm,
                 long long timeout_ns, GeoTab<N> gt)
{
    static_assert(!GEO || (OP == OP_RES && MG && sizeof(T) == 4), "on-the-fly geometry: FP32 Res, two components");
    constexpr int NN = N * N;
    constexpr int NC = op_nc<OP>();
    constexpr int NA = bulk_arrays_g<OP, GEO>();
    constexpr int K = bulk_k<T, OP>(N);
    constexpr int BN = K * NN;
    constexpr int S = BULK_STAGES;
    extern __shared__ __align__(128) unsigned char smb[];
    uint64_t* bar = (uint64_t*)smb;
    T* stage0 = (T*)(smb + 128);
    T* W1 = stage0 + (size_t)S * NA * BN;
    T* W2 = W1 + NC * BN;
    float* geo0 = (float*)(W2 + NC * BN);  // GEO: per stage K * GEO_PER_EL corner differences
    const Fac<T> fac = fac_of<T>(m);
    const T* arr[7];
    {
        int a = 0;
        arr[a++] = in0;
        if (NC == 2) arr[a++] = in1;
        if (!GEO) {
            if (OP != OP_MASS) {
                arr[a++] = fac.g11;
                arr[a++] = fac.g12;
                arr[a++] = fac.g22;
            }
            if (OP != OP_LAPLACE) arr[a++] = fac.mass;
        }
        if (OP == OP_HELM || OP == OP_RES || OP == OP_F) arr[a++] = pot;
    }
    T* outp[2] = {y0, y1};
    constexpr int A_G11 = NC, A_MASS = (OP == OP_MASS) ? NC : NC + 3, A_POT = GEO ? NC : A_MASS + 1;
    const long long nfull = m.E / K;  // batches loaded by bulk copies
    const long long nbatch = (m.E + K - 1) / K;
    const long long G = gridDim.x;
    uint32_t pending = 0;  // thread 0: stages with a copy in flight
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    auto issue = [&](long long b, int s) {  // thread 0 only
        if (b >= nfull) return;
        T* st = stage0 + (size_t)s * NA * BN;
        constexpr uint32_t bytes = (uint32_t)(BN * sizeof(T));
        constexpr uint32_t gbytes = GEO ? (uint32_t)(K * GEO_PER_EL * sizeof(float)) : 0u;
        mbar_arrive_tx(&bar[s], bytes * NA + gbytes);
#pragma unroll
        for (int a = 0; a < NA; ++a) bulk_load(st + a * BN, arr[a] + b * BN, bytes, &bar[s]);
        if (GEO) bulk_load(geo0 + (size_t)s * K * GEO_PER_EL, m.geo32 + b * K * GEO_PER_EL, gbytes, &bar[s]);
        pending |= 1u << s;
    };
    if (threadIdx.x == 0)
        for (int s = 0; s < S; ++s) issue(blockIdx.x + s * G, s);
    // masked input: ring copies that are not the owner take the owner's value
    // (ring_src).  The table entries of a block's batches are loaded two
    // batches ahead and the owner values one batch ahead, so neither load
    // is waited for while the batch that needs it is still to come.
    constexpr int R = 4 * (N - 1);
    constexpr int TPB = bulk_tpb_k<T, OP, MG>();
    constexpr int GQ = (K * R + TPB - 1) / TPB;
    int gsrc[GQ], gsrc_n[GQ], gsrc_nn[GQ];  // tables of batches b, b+G, b+2G
    T gval[GQ][NC], gval_n[GQ][NC];         // owner values of batches b, b+G
    auto gather_tab = [&](long long bb, int (&dst)[GQ]) {
        const int neb = bb < nbatch ? min(K, m.E - (int)(bb * K)) : 0;
        const int nr = neb * R;
        const int* rs = m.ring_src + bb * K * R;
#pragma unroll
        for (int q = 0; q < GQ; ++q) {
            const int t = threadIdx.x + q * TPB;
            dst[q] = t < nr ? __ldg(rs + t) : -1;
        }
    };
    auto gather_val = [&](const int (&src)[GQ], T (&dst)[GQ][NC]) {
#pragma unroll
        for (int q = 0; q < GQ; ++q)
            if (src[q] >= 0) {
#pragma unroll
                for (int c = 0; c < NC; ++c) dst[q][c] = arr[c][src[q]];
            }
    };
    auto gather_apply = [&](T* st, int ne) {
#pragma unroll
        for (int q = 0; q < GQ; ++q) {
            if (gsrc[q] < 0) continue;
            const int t = threadIdx.x + q * TPB;
            const int le = t / R;
            const int r = t - le * R;
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
#pragma unroll
            for (int c = 0; c < NC; ++c) st[c * BN + le * NN + ii + jj * N] = gval[q][c];
        }
    };
    // side pairs with both copies in the batch (pair_asm): owner += other,
    // other = 0 in the staged result, before it is stored.  Range of a batch's
    // entries loaded two batches ahead, the entries one batch ahead.
    constexpr int PQ = (2 * K * (N - 2) + TPB - 1) / TPB > 0 ? (2 * K * (N - 2) + TPB - 1) / TPB : 1;
    int ppair[PQ], ppair_n[PQ];
    int2 prng_n = make_int2(0, 0), prng_nn = make_int2(0, 0);  // entry ranges of batches b+G, b+2G
    auto pair_rng = [&](long long bb) {
        int2 r = make_int2(0, 0);
        if (pair_asm && bb < nbatch) {
            r.x = __ldg(m.bulk_pair_ptr + bb);
            r.y = __ldg(m.bulk_pair_ptr + bb + 1);
        }
        return r;
    };
    auto pair_ent = [&](int2 r, int (&dst)[PQ]) {
        if (threadIdx.x == 0 && r.y - r.x > PQ * TPB) atomicExch(m.dev_err, 2);  // cannot happen: <= 2K(N-2)
#pragma unroll
        for (int q = 0; q < PQ; ++q) {
            const int t = r.x + threadIdx.x + q * TPB;
            dst[q] = t < r.y ? __ldg(m.bulk_pairs + t) : -1;
        }
    };
    if (GATHER) {
        gather_tab(blockIdx.x, gsrc);
        gather_val(gsrc, gval);
        gather_tab(blockIdx.x + G, gsrc_n);
    }
    pair_ent(pair_rng(blockIdx.x), ppair);
    prng_n = pair_rng(blockIdx.x + G);
    int it = 0;
    for (long long b = blockIdx.x; b < nbatch; b += G, ++it) {
        const int s = it % S;
        const uint32_t parity = (uint32_t)((it / S) & 1);
        T* st = stage0 + (size_t)s * NA * BN;
        const int e0 = (int)(b * K);
        const int ne = min(K, m.E - e0);
        const int total = ne * NN;
        bool ok = true;
        if (b < nfull) {
            ok = mbar_wait(&bar[s], parity, timeout_ns);
        } else {
            for (int t = threadIdx.x; t < total; t += blockDim.x)
#pragma unroll
                for (int a = 0; a < NA; ++a) st[a * BN + t] = arr[a][(long long)e0 * NN + t];
            if (GEO)
                for (int t = threadIdx.x; t < ne * GEO_PER_EL; t += blockDim.x)
                    geo0[(size_t)s * K * GEO_PER_EL + t] = m.geo32[(long long)e0 * GEO_PER_EL + t];
        }
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0) {
                atomicExch(m.dev_err, 1);
                for (int q = 1; q < S; ++q) {  // copies of the other stages still in flight (bounded)
                    const int sq = (s + q) % S;
                    if (pending & (1u << sq)) mbar_wait(&bar[sq], (uint32_t)(((it + q) / S) & 1), timeout_ns);
                }
                bulk_wait_all();
            }
            __syncthreads();
            return;
        }
        if (threadIdx.x == 0) pending &= ~(1u << s);
        if (GATHER) {
            gather_apply(st, ne);
            __syncthreads();
            gather_val(gsrc_n, gval_n);  // in flight while this batch computes
            gather_tab(b + 2 * G, gsrc_nn);
        }
        if (pair_asm) {
            pair_ent(prng_n, ppair_n);
            prng_nn = pair_rng(b + 2 * G);
        }
        if (OP == OP_MASS) {
            for (int t = threadIdx.x; t < total; t += blockDim.x) y0[(long long)e0 * NN + t] = st[A_MASS * BN + t] * st[t];
        } else if constexpr (MG) {
            // Res, both components per thread: thread t works on line t
            const int l0 = threadIdx.x;
            const bool act = l0 < ne * N;
            const int le = l0 / N, l = l0 - (l0 / N) * N;
            const int base = le * NN;
            GeoLine gl{};
            if constexpr (GEO) gl = geo_line<N>(gt, l);
            T* w1a = W1 + base;
            T* w1b = W1 + BN + base;
            T* w2a = W2 + base;
            T* w2b = W2 + BN + base;
            if (threadIdx.x == 0 && store_bulk) bulk_wait_read();
            __syncthreads();
            T ura[N], urb[N];
            // ---- P1: column l -> ur (registers); row l -> us (W1)
            if (act) {
                const T* ua = st + base;
                const T* ub = st + BN + base;
                T va[N], vb[N], aa[N], ab[N];
#pragma unroll
                for (int i = 0; i < N; ++i) {
                    va[i] = ua[l * N + i];
                    vb[i] = ub[l * N + i];
                    ura[i] = T(0);
                    urb[i] = T(0);
                }
                contract2<N, false, bulk_f2(N)>(D, D2, va, vb, ura, urb);
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    va[j] = ua[j * N + l];
                    vb[j] = ub[j * N + l];
                    aa[j] = T(0);
                    ab[j] = T(0);
                }
                contract2<N, false, bulk_f2(N)>(D, D2, va, vb, aa, ab);
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    w1a[j * N + l] = aa[j];
                    w1b[j * N + l] = ab[j];
                }
            }
            __syncthreads();
            // ---- P2: column l: fluxes (factors read once); f2 -> W1, lap1 = D^T f1 -> W2
            if (act) {
                T fa[N], fb[N], aa[N], ab[N];
                float gq[GEO_PER_EL];
                if (GEO) {
#pragma unroll
                    for (int k = 0; k < GEO_PER_EL; ++k) gq[k] = geo0[((size_t)s * K + le) * GEO_PER_EL + k];
                }
#pragma unroll
                for (int i = 0; i < N; ++i) {
                    const int q = base + l * N + i;
                    T g11, g12, g22;
                    if constexpr (GEO) {
                        geo_factors_col<N>(gt, gq, i, gl, g11, g12, g22);
                    } else {
                        g11 = st[A_G11 * BN + q];
                        g12 = st[(A_G11 + 1) * BN + q];
                        g22 = st[(A_G11 + 2) * BN + q];
                    }
                    const T usa = w1a[l * N + i], usb = w1b[l * N + i];
                    fa[i] = g11 * ura[i] - g12 * usa;
                    fb[i] = g11 * urb[i] - g12 * usb;
                    w1a[l * N + i] = g22 * usa - g12 * ura[i];
                    w1b[l * N + i] = g22 * usb - g12 * urb[i];
                    aa[i] = T(0);
                    ab[i] = T(0);
                }
                contract2<N, true, bulk_f2(N)>(D, D2, fa, fb, aa, ab);
#pragma unroll
                for (int i = 0; i < N; ++i) {
                    w2a[l * N + i] = aa[i];
                    w2b[l * N + i] = ab[i];
                }
            }
            __syncthreads();
            // ---- P3: row l: lap = lap1 + f2 D for both components, then the
            // Res combination -> W1 (row l of W1 is read and written by this
            // thread only)
            if (act) {
                T la[N], lb[N], fa[N], fb[N];
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    la[j] = w2a[j * N + l];
                    lb[j] = w2b[j * N + l];
                    fa[j] = w1a[j * N + l];
                    fb[j] = w1b[j * N + l];
                }
                contract2<N, true, bulk_f2(N)>(D, D2, fa, fb, la, lb);
                float gq[GEO_PER_EL];
                if (GEO) {
#pragma unroll
                    for (int k = 0; k < GEO_PER_EL; ++k) gq[k] = geo0[((size_t)s * K + le) * GEO_PER_EL + k];
                }
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    const int q = base + j * N + l;
                    T ms;
                    if constexpr (GEO) {
                        ms = geo_mass_row<N>(gt, gq, gl, j);
                    } else {
                        ms = st[A_MASS * BN + q];
                    }
                    const T pv = st[A_POT * BN + q];
                    const T mv = ms * pv;
                    const T u0 = st[q], u1 = st[BN + q];
                    const T lap0 = la[j], lap1 = lb[j];
                    const T Lv = lap1 + mv * u1;
                    const T Lu = lap0 + mv * u0;
                    W1[q] = ms * u0 + alpha * Lv;
                    W1[BN + q] = alpha * Lu - ms * u1;
                }
            }
        } else {
            // thread t works on component c = t / LP, line t % LP
            constexpr int LP = TPB / NC;
            const int c = threadIdx.x / LP;
            const int line = threadIdx.x - c * LP;
            const bool act = line < ne * N;
            const int le = line / N, l = line - (line / N) * N;
            const int base = le * NN;
            T* w1 = W1 + c * BN + base;
            T* w2 = W2 + c * BN + base;
            // W1 is written below and was the previous batch's bulk-store source
            if (threadIdx.x == 0 && store_bulk) bulk_wait_read();
            __syncthreads();
            T ur[N];
            // ---- P1: column l -> ur (registers); row l -> us (W1)
            if (act) {
                const T* uc = st + c * BN + base;
                T v[N], acc[N];
#pragma unroll
                for (int i = 0; i < N; ++i) {
                    v[i] = uc[l * N + i];
                    ur[i] = T(0);
                }
#pragma unroll
                for (int k = 0; k < N; ++k)
#pragma unroll
                    for (int i = 0; i < N; ++i) ur[i] = fma(D.d[i * N + k], v[k], ur[i]);
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    v[j] = uc[j * N + l];
                    acc[j] = T(0);
                }
#pragma unroll
                for (int k = 0; k < N; ++k)
#pragma unroll
                    for (int j = 0; j < N; ++j) acc[j] = fma(D.d[j * N + k], v[k], acc[j]);
#pragma unroll
                for (int j = 0; j < N; ++j) w1[j * N + l] = acc[j];
            }
            __syncthreads();
            // ---- P2: column l: fluxes; f2 -> W1, lap1 = D^T f1 -> W2
            if (act) {
                T f1[N], acc[N];
#pragma unroll
                for (int i = 0; i < N; ++i) {
                    const int q = base + l * N + i;
                    const T g11 = st[A_G11 * BN + q], g12 = st[(A_G11 + 1) * BN + q], g22 = st[(A_G11 + 2) * BN + q];
                    const T us = w1[l * N + i];
                    f1[i] = g11 * ur[i] - g12 * us;
                    w1[l * N + i] = g22 * us - g12 * ur[i];
                    acc[i] = T(0);
                }
#pragma unroll
                for (int k = 0; k < N; ++k)
#pragma unroll
                    for (int i = 0; i < N; ++i) acc[i] = fma(D.d[k * N + i], f1[k], acc[i]);
#pragma unroll
                for (int i = 0; i < N; ++i) w2[l * N + i] = acc[i];
            }
            __syncthreads();
            // ---- P3: row l: lap = lap1 + f2 D -> W2 (in place)
            if (act) {
                T lap[N], f2[N];
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    lap[j] = w2[j * N + l];
                    f2[j] = w1[j * N + l];
                }
#pragma unroll
                for (int k = 0; k < N; ++k)
#pragma unroll
                    for (int j = 0; j < N; ++j) lap[j] = fma(D.d[k * N + j], f2[k], lap[j]);
#pragma unroll
                for (int j = 0; j < N; ++j) w2[j * N + l] = lap[j];
            }
            __syncthreads();
            // ---- P4: row l, component c of the operator (the Res/f
            // combination reads the other component's laplacian) -> W1
            if (act) {
#pragma unroll
                for (int j = 0; j < N; ++j) {
                    const int q = base + j * N + l;
                    T o;
                    if (OP == OP_LAPLACE) {
                        o = W2[q];
                    } else {
                        const T ms = st[A_MASS * BN + q];
                        const T pv = (OP == OP_HELM || OP == OP_RES || OP == OP_F) ? st[A_POT * BN + q] : T(0);
                        if (OP == OP_HELM) {
                            o = W2[q] + (ms * pv) * st[q];
                        } else {
                            const T mv = ms * pv;
                            const T u0 = st[q], u1 = st[(NC - 1) * BN + q];
                            const T lap0 = W2[q], lap1 = W2[(NC - 1) * BN + q];
                            if (OP == OP_RES) {
                                if (c == 0) {
                                    const T Lv = lap1 + mv * u1;
                                    o = ms * u0 + alpha * Lv;
                                } else {
                                    const T Lu = lap0 + mv * u0;
                                    o = alpha * Lu - ms * u1;
                                }
                            } else {  // OP_F
                                o = (c == 0) ? -(lap1 + mv * u1) : -(lap0 + mv * u0);
                            }
                        }
                    }
                    W1[c * BN + q] = o;
                }
            }
        }
        if (OP != OP_MASS) {  // the staged result (W1): batch-internal side pairs, then the store
            if (pair_asm) {
                __syncthreads();
#pragma unroll
                for (int q = 0; q < PQ; ++q) {
                    if (ppair[q] < 0) continue;
                    const int po = ppair[q] >> 16, px = ppair[q] & 0xffff;
#pragma unroll
                    for (int cc = 0; cc < NC; ++cc) {
                        W1[cc * BN + po] = W1[cc * BN + po] + W1[cc * BN + px];  // owner + other, as k_ring
                        W1[cc * BN + px] = T(0);
                    }
                }
            }
            fence_proxy_async_smem();
            __syncthreads();
            if (store_bulk && b < nfull) {
                if (threadIdx.x == 0) {
#pragma unroll
                    for (int cc = 0; cc < NC; ++cc)
                        bulk_store(outp[cc] + (long long)e0 * NN, W1 + cc * BN, (uint32_t)(BN * sizeof(T)));
                    bulk_commit();
                }
            } else {
                for (int t = threadIdx.x; t < total; t += blockDim.x)
#pragma unroll
                    for (int cc = 0; cc < NC; ++cc) outp[cc][(long long)e0 * NN + t] = W1[cc * BN + t];
            }
        }
        // the next batch's tables and values (loaded during this one)
        if (GATHER) {
#pragma unroll
            for (int q = 0; q < GQ; ++q) {
                gsrc[q] = gsrc_n[q];
                gsrc_n[q] = gsrc_nn[q];
#pragma unroll
                for (int c = 0; c < NC; ++c) gval[q][c] = gval_n[q][c];
            }
        }
        if (pair_asm) {
#pragma unroll
            for (int q = 0; q < PQ; ++q) ppair[q] = ppair_n[q];
            prng_n = prng_nn;
        }
        // stage s free; this thread's shared-memory accesses ordered before
        // the bulk copy that refills it
        fence_proxy_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) issue(b + (long long)S * G, s);
    }
    if (threadIdx.x == 0) bulk_wait_all();
}

// grid of k_apply_bulk for one instantiation.  The shared-memory opt-in is
// a per-device attribute, so it is set, and the occupancy queried, once per
// device (the current one, which owns the launch's stream), under a lock.
template <int N, typename T, int OP, bool GATHER, bool MG, bool GEO>
cudaError_t launch_apply_bulk_mg(const DevMesh& m, const T* pot, T alpha, const T* in0, const T* in1, T* y0, T* y1,
                                 bool pair_asm, long long timeout_ns, cudaStream_t st)
{
    constexpr int kMaxDev = 64;
    static std::mutex mu;
    static bool ready[kMaxDev] = {};
    static int blocks_per_sm_of[kMaxDev] = {}, sms_of[kMaxDev] = {};
    constexpr size_t smem = bulk_smem_bytes<N, T, OP, GEO>();
    constexpr int TPB = bulk_tpb_k<T, OP, MG>();
    const auto kern = k_apply_bulk<N, T, OP, GATHER, MG, GEO>;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    int blocks_per_sm = 0, sms = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!ready[dev]) {
            e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            if ((e = cudaDeviceGetAttribute(&sms_of[dev], cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
                return e;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm_of[dev], kern, TPB, smem)) !=
                cudaSuccess)
                return e;
            ready[dev] = true;
        }
        blocks_per_sm = blocks_per_sm_of[dev];
        sms = sms_of[dev];
    }
    if (blocks_per_sm < 1) return cudaErrorInvalidConfiguration;
    if (!m.Dh) return cudaErrorInvalidValue;
    if (GEO && (!m.geo32 || !m.zh || !m.wh)) return cudaErrorInvalidValue;
    DMat<N, T> D;
    DMat2<N> D2 = {};
    for (int i = 0; i < N * N; ++i) {
        D.d[i] = (T)m.Dh[i];
        if (MG) {
            const float f = (float)m.Dh[i];
            uint32_t u;
            memcpy(&u, &f, sizeof(u));
            D2.d[i] = ((unsigned long long)u << 32) | u;
        }
    }
    GeoTab<N> gt = {};
    if (GEO) {
        for (int i = 0; i < N; ++i) {
            gt.lo[i] = (float)(0.25 * (1.0 - m.zh[i]));
            gt.hi[i] = (float)(0.25 * (1.0 + m.zh[i]));
            gt.w[i] = (float)m.wh[i];
        }
        gt.corrected = m.corrected;
    }
    constexpr int K = bulk_k<T, OP>(N);
    const long long nbatch = (m.E + K - 1) / K;
    const int grid = (int)std::min<long long>(nbatch, (long long)sms * blocks_per_sm);
    const int store_bulk = (((uintptr_t)y0 | (uintptr_t)(y1 ? y1 : y0)) & 15u) == 0;
    // batch-local pair tables exist for the FP32 Res batching only
    const int pa = (pair_asm && OP == OP_RES && sizeof(T) == 4 && m.bulk_K == K && m.bulk_pair_ptr) ? 1 : 0;
    if (pair_asm && !pa) return cudaErrorInvalidValue;
    kern<<<grid, TPB, smem, st>>>(m, D, D2, pot, alpha, in0, in1, y0, y1, store_bulk, pa, timeout_ns, gt);
    return cudaGetLastError();
}

// Res with both components per thread, by degree: the FP32 sweep at about
// 20 M nodes (L2 flushed) ran it 12-36 % faster for p = 2..11, 14 and 15 and
// 3-10 % slower for p = 12, 13 and 16, where the batches hold only 4
// elements and most of its threads have no line
__host__ __device__ constexpr bool bulk_mg(int N) { return !(N == 13 || N == 14 || N == 17); }

// geo: the geometric factors computed on the fly from the element corners
// (FP32 Res with both components per thread); otherwise they are read
template <int N, typename T, int OP, bool GATHER>
cudaError_t launch_apply_bulk_t(const DevMesh& m, const T* pot, T alpha, const T* in0, const T* in1, T* y0, T* y1,
                                bool pair_asm, bool geo, long long timeout_ns, cudaStream_t st)
{
    constexpr bool MG = OP == OP_RES && bulk_mg(N);
    if constexpr (MG && sizeof(T) == 4) {
        if (geo)
            return launch_apply_bulk_mg<N, T, OP, GATHER, MG, true>(m, pot, alpha, in0, in1, y0, y1, pair_asm,
                                                                    timeout_ns, st);
    }
    return launch_apply_bulk_mg<N, T, OP, GATHER, MG, false>(m, pot, alpha, in0, in1, y0, y1, pair_asm, timeout_ns,
                                                             st);
}

}  // namespace semgb
