// Learned initial guess for the implicit stage solves: a per-element MLP
// (BF16 weights and activations on the tensor cores, FP32 accumulation,
// FP32 master weights and Adam state) trained on the GPU with this file's
// own forward and backward kernels.
//
// Model: x (d_in) -> ReLU(x W1 + b1) (H) -> ReLU(. W2 + b2) (H) -> . W3 + b3 (d_out)
// with row-major activations [rows][features] and weights [in][out].
//
// GEMM: C[M][N] = A(M x K) * B(K x N) with generic strides, tiles of 64 x 64
// staged in shared memory as BF16, computed with mma.sync m16n8k16 (BF16 in,
// FP32 accumulate); every global access is bounds-checked.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "sem_gb300.h"
#include "sem_apply_bulk.cuh"  // mbarrier helpers
#include "sem_device.cuh"
#include "sem_internal.h"

using namespace semgb;

namespace {

constexpr int GT_M = 64, GT_N = 64, GT_K = 32;

struct GemmArgs {
    int M, N, K;
    const void* A;
    long long sa_m, sa_k;  // A(m,k) = A[m*sa_m + k*sa_k]
    int a_bf16;            // A is __nv_bfloat16 (else float)
    const void* B;
    long long sb_k, sb_n;  // B(k,n) = B[k*sb_k + n*sb_n]
    int b_bf16;
    float* C;              // C[m*ldc + n] (FP32)
    int ldc;
    const float* bias;     // optional, length N
    int relu;              // ReLU epilogue
    int accumulate;        // C += result
    __nv_bfloat16* Cbf;    // optional BF16 copy of the output
};

__device__ __forceinline__ float ld_any(const void* p, long long i, int bf)
{
    return bf ? __bfloat162float(((const __nv_bfloat16*)p)[i]) : ((const float*)p)[i];
}

__device__ __forceinline__ uint32_t pack_bf16(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// 128 threads = 4 warps in a 2 x 2 arrangement, each warp 32 x 32 of C
__global__ void __launch_bounds__(128) k_gemm_bf16(GemmArgs g)
{
    // A tile [64][32] and B tile transposed [64 n][32 k], BF16, padded rows
    __shared__ __nv_bfloat16 sA[GT_M][GT_K + 8];
    __shared__ __nv_bfloat16 sB[GT_N][GT_K + 8];
    const int m0 = blockIdx.y * GT_M, n0 = blockIdx.x * GT_N;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][b][c] = 0.f;
    const int gq = lane >> 2, tq = lane & 3;  // mma fragment coordinates
    for (int k0 = 0; k0 < g.K; k0 += GT_K) {
        for (int t = threadIdx.x; t < GT_M * GT_K; t += blockDim.x) {
            const int r = t / GT_K, c = t - r * GT_K;
            const int m = m0 + r, k = k0 + c;
            const float v = (m < g.M && k < g.K) ? ld_any(g.A, m * g.sa_m + k * g.sa_k, g.a_bf16) : 0.f;
            sA[r][c] = __float2bfloat16(v);
        }
        for (int t = threadIdx.x; t < GT_N * GT_K; t += blockDim.x) {
            const int r = t / GT_K, c = t - r * GT_K;  // r: n, c: k
            const int n = n0 + r, k = k0 + c;
            const float v = (n < g.N && k < g.K) ? ld_any(g.B, k * g.sb_k + n * g.sb_n, g.b_bf16) : 0.f;
            sB[r][c] = __float2bfloat16(v);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GT_K; kk += 16) {
            uint32_t af[2][4], bfr[4][2];
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                const int r = wm + a * 16 + gq;
                af[a][0] = pack_bf16(sA[r][kk + 2 * tq], sA[r][kk + 2 * tq + 1]);
                af[a][1] = pack_bf16(sA[r + 8][kk + 2 * tq], sA[r + 8][kk + 2 * tq + 1]);
                af[a][2] = pack_bf16(sA[r][kk + 2 * tq + 8], sA[r][kk + 2 * tq + 9]);
                af[a][3] = pack_bf16(sA[r + 8][kk + 2 * tq + 8], sA[r + 8][kk + 2 * tq + 9]);
            }
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int nn = wn + b * 8 + gq;
                bfr[b][0] = pack_bf16(sB[nn][kk + 2 * tq], sB[nn][kk + 2 * tq + 1]);
                bfr[b][1] = pack_bf16(sB[nn][kk + 2 * tq + 8], sB[nn][kk + 2 * tq + 9]);
            }
#pragma unroll
            for (int a = 0; a < 2; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b)
                    asm volatile(
                        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
                        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                        : "+f"(acc[a][b][0]), "+f"(acc[a][b][1]), "+f"(acc[a][b][2]), "+f"(acc[a][b][3])
                        : "r"(af[a][0]), "r"(af[a][1]), "r"(af[a][2]), "r"(af[a][3]), "r"(bfr[b][0]),
                          "r"(bfr[b][1]));
        }
        __syncthreads();
    }
    // epilogue: fragment (row gq / gq+8, cols 2tq, 2tq+1)
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int m = m0 + wm + a * 16 + gq + h * 8;
                    const int nn = n0 + wn + b * 8 + 2 * tq + q;
                    if (m >= g.M || nn >= g.N) continue;
                    float v = acc[a][b][h * 2 + q];
                    if (g.accumulate) v += g.C[(long long)m * g.ldc + nn];
                    if (g.bias) v += g.bias[nn];
                    if (g.relu) v = fmaxf(v, 0.f);
                    g.C[(long long)m * g.ldc + nn] = v;
                    if (g.Cbf) g.Cbf[(long long)m * g.ldc + nn] = __float2bfloat16(v);
                }
}

// ------------------------------------------------ tcgen05 (5th-generation) GEMM
// The same GEMM on the sm_100-family tensor cores: tcgen05.mma kind::f16
// (BF16 A and B, FP32 accumulator in tensor memory), M = 128 rows per CTA,
// N = TC_BN columns, K in steps of 16 from shared-memory operands staged by
// the CTA's 128 threads (generic strides, FP32 or BF16 sources converted to
// BF16, zero-filled past the matrix edges) in the canonical K-major layout
// without swizzle: 8-row x 16-byte core matrices, the two core matrices of a
// 16-wide K step 128 bytes apart (leading-dimension offset), consecutive
// 8-row groups 256 bytes apart (stride-dimension offset).  Two K tiles of 64
// are staged alternately: the loads of tile k+1 overlap the MMAs of tile k,
// and a tile's buffer is reused only after the mbarrier its commit arrives on
// has completed.  One thread issues the MMAs; the four warps then read the
// accumulator rows they own (TMEM lanes 32w..32w+31) with tcgen05.ld and run
// the epilogue.  Every wait is bounded; the CTA always frees its tensor
// memory before it returns.
constexpr int TC_M = 128, TC_BK = 64, TC_THREADS = 128;
__device__ int g_tc_err;  // set when a bounded wait of k_gemm_tc expired

__host__ __device__ constexpr uint32_t tc_idesc(int m, int n)
{
    return (1u << 4)                         // accumulator: FP32
           | (1u << 7)                       // A: BF16
           | (1u << 10)                      // B: BF16 (both K-major, not negated)
           | ((uint32_t)(n >> 3) << 17)      // N / 8
           | ((uint32_t)(m >> 4) << 24);     // M / 16
}

__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);  // version 1, no swizzle
}

// byte offset of (row r, k) in a staged tile of R rows x TC_BK
__device__ __forceinline__ uint32_t tc_off(int R, int r, int k)
{
    return (uint32_t)((k >> 4) * (R * 32) + (r >> 3) * 256 + ((k >> 3) & 1) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// 8 consecutive values of one operand row (K-contiguous when stride 1),
// packed as 4 BF16 pairs; vector loads when the row run is aligned and in range
__device__ __forceinline__ void tc_chunk(const void* X, int bf, long long base, long long sk, int kvalid,
                                         uint32_t (&w)[4])
{
    if (sk == 1 && kvalid >= 8) {
        if (bf) {
            const __nv_bfloat16* p = (const __nv_bfloat16*)X + base;
            const uintptr_t a = (uintptr_t)p;
            if ((a & 15) == 0) {
                const uint4 v = __ldg((const uint4*)p);
                w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
                return;
            }
            if ((a & 7) == 0) {
                const uint2 v0 = __ldg((const uint2*)p), v1 = __ldg((const uint2*)p + 1);
                w[0] = v0.x; w[1] = v0.y; w[2] = v1.x; w[3] = v1.y;
                return;
            }
            if ((a & 3) == 0) {
#pragma unroll
                for (int h = 0; h < 4; ++h) w[h] = __ldg((const unsigned int*)p + h);
                return;
            }
        } else {
            const float* p = (const float*)X + base;
            if (((uintptr_t)p & 15) == 0) {
                const float4 v0 = __ldg((const float4*)p), v1 = __ldg((const float4*)p + 1);
                w[0] = pack_bf16(__float2bfloat16(v0.x), __float2bfloat16(v0.y));
                w[1] = pack_bf16(__float2bfloat16(v0.z), __float2bfloat16(v0.w));
                w[2] = pack_bf16(__float2bfloat16(v1.x), __float2bfloat16(v1.y));
                w[3] = pack_bf16(__float2bfloat16(v1.z), __float2bfloat16(v1.w));
                return;
            }
        }
    }
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        const float v0 = (2 * h < kvalid) ? ld_any(X, base + (long long)(2 * h) * sk, bf) : 0.f;
        const float v1 = (2 * h + 1 < kvalid) ? ld_any(X, base + (long long)(2 * h + 1) * sk, bf) : 0.f;
        w[h] = pack_bf16(__float2bfloat16(v0), __float2bfloat16(v1));
    }
}

template <int BN>
__device__ __forceinline__ void tc_stage(const GemmArgs& g, unsigned char* sA, unsigned char* sB, int m0, int n0,
                                         int k0)
{
    // 16-byte chunks: 8 consecutive k of one row; every thread issues all of
    // its chunks' loads before its shared-memory stores
    constexpr int NQ = ((TC_M + BN) * (TC_BK / 8) + TC_THREADS - 1) / TC_THREADS;
    uint32_t w[NQ][4];
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
        const int q = threadIdx.x + i * TC_THREADS;
        const bool isA = q < TC_M * (TC_BK / 8);
        const int qq = isA ? q : q - TC_M * (TC_BK / 8);
        const int r = qq >> 3, kc = qq & 7;
        const int k = k0 + kc * 8;
        const int row = (isA ? m0 : n0) + r;
        const bool in = isA ? (row < g.M) : (row < g.N);
        const int kvalid = in ? min(8, g.K - k) : 0;
        if (kvalid <= 0) {
            w[i][0] = w[i][1] = w[i][2] = w[i][3] = 0u;
            continue;
        }
        if (isA)
            tc_chunk(g.A, g.a_bf16, (long long)row * g.sa_m + (long long)k * g.sa_k, g.sa_k, kvalid, w[i]);
        else
            tc_chunk(g.B, g.b_bf16, (long long)k * g.sb_k + (long long)row * g.sb_n, g.sb_k, kvalid, w[i]);
    }
#pragma unroll
    for (int i = 0; i < NQ; ++i) {
        const int q = threadIdx.x + i * TC_THREADS;
        const bool isA = q < TC_M * (TC_BK / 8);
        const int qq = isA ? q : q - TC_M * (TC_BK / 8);
        const int r = qq >> 3, kc = qq & 7;
        unsigned char* dst = (isA ? sA + tc_off(TC_M, r, kc * 8) : sB + tc_off(BN, r, kc * 8));
        *(uint4*)dst = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
    }
}

template <int BN>
__global__ void __launch_bounds__(TC_THREADS) k_gemm_tc(GemmArgs g, long long timeout_ns)
{
    extern __shared__ __align__(1024) unsigned char tsm[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tmem_base;
    constexpr int ABYTES = TC_M * TC_BK * 2, BBYTES = BN * TC_BK * 2;
    // stage b: A tile at tsm + b (ABYTES + BBYTES), its B tile right after
    auto sA = [&](int b) { return tsm + (size_t)b * (ABYTES + BBYTES); };
    auto sB = [&](int b) { return tsm + (size_t)b * (ABYTES + BBYTES) + ABYTES; };
    const int m0 = blockIdx.y * TC_M, n0 = blockIdx.x * BN;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = tmem_base;
    constexpr uint32_t idesc = tc_idesc(TC_M, BN);
    const int nk = (g.K + TC_BK - 1) / TC_BK;
    bool ok = true;
    int issued = 0;  // K chunks whose MMAs thread 0 has committed
    for (int kt = 0; kt < nk && ok; ++kt) {
        const int b = kt & 1;
        if (kt >= 2) ok = mbar_wait(&bar[b], (uint32_t)(((kt - 2) >> 1) & 1), timeout_ns);
        if (!__syncthreads_and(ok)) {
            ok = false;
            break;
        }
        tc_stage<BN>(g, sA(b), sB(b), m0, n0, kt * TC_BK);
        fence_proxy_async_smem();  // the staged tile is read by the tensor cores (async proxy)
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = smem_addr(sA(b)), b0 = smem_addr(sB(b));
#pragma unroll
            for (int ks = 0; ks < TC_BK / 16; ++ks) {
                const uint64_t ad = tc_desc(a0 + ks * TC_M * 32, 128, 256);
                const uint64_t bd = tc_desc(b0 + ks * BN * 32, 128, 256);
                const uint32_t acc = (kt > 0 || ks > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(taddr),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(&bar[b]))
                         : "memory");
        }
        issued = kt + 1;
    }
    if (ok && nk > 0) ok = mbar_wait(&bar[(nk - 1) & 1], (uint32_t)(((nk - 1) >> 1) & 1), timeout_ns);
    ok = __syncthreads_and(ok) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        const int m = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            uint32_t r[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (m < g.M) {
                // every load of the chunk (bias, accumulated C) before its
                // first store: the stores may alias them as far as the
                // compiler knows, which would serialise load after store
                float cin[16], bin[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int nn = n0 + c0 + j;
                    const bool in = nn < g.N;
                    cin[j] = (in && g.accumulate) ? g.C[(long long)m * g.ldc + nn] : 0.f;
                    bin[j] = (in && g.bias) ? __ldg(g.bias + nn) : 0.f;
                }
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int nn = n0 + c0 + j;
                    if (nn >= g.N) continue;
                    float v = __uint_as_float(r[j]);
                    if (g.accumulate) v += cin[j];
                    if (g.bias) v += bin[j];
                    if (g.relu) v = fmaxf(v, 0.f);
                    g.C[(long long)m * g.ldc + nn] = v;
                    if (g.Cbf) g.Cbf[(long long)m * g.ldc + nn] = __float2bfloat16(v);
                }
            }
        }
    } else {
        if (threadIdx.x == 0) atomicExch(&g_tc_err, 1);
        // a wait ran out: give the MMAs already committed (the last commit
        // covers every earlier one) one more bounded wait before the
        // accumulator's tensor memory is freed
        if (issued > 0) mbar_wait(&bar[(issued - 1) & 1], (uint32_t)(((issued - 1) >> 1) & 1), timeout_ns);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(BN) : "memory");
}

// ------------------------------------------------ fused forward pass
// The network's inference pass in one kernel: per CTA 128 rows, the three
// layers chained through tensor memory and shared memory.  Layer 1 streams
// its A tile (the BF16 features) and every layer streams its weights
// (transposed BF16 copies, K contiguous) in 64-wide K chunks through two
// shared-memory buffers; the hidden activations never leave the SM: the
// epilogue of layers 1 and 2 reads the FP32 accumulator with tcgen05.ld,
// adds the bias, applies ReLU, rounds to BF16 and writes them in the
// canonical K-major layout as the next layer's A operand (H, all 256 K at
// once).  Accumulators: layer 1 in TMEM columns [0, H), layer 2 in
// [256, 256 + H), layer 3 in [0, d_out rounded up to 16).  Same BF16
// rounding points and MMA shapes as the per-layer GEMMs (M = 128, K = 16
// steps in order), so the results agree with them.  Shapes: H <= 256 and
// H, d_out <= 256; otherwise the per-layer GEMMs run.
constexpr int MF_BUF = 48 * 1024;  // one staging buffer: A chunk (16 KB) + B chunk (<= 32 KB)
constexpr int MF_H = 64 * 1024;    // hidden activations, 128 rows x 256 K BF16
constexpr size_t MF_SMEM = 2 * (size_t)MF_BUF + MF_H;

struct MlpArgs {
    int rows, d_in, H, d_out;
    const __nv_bfloat16* x;       // rows x d_in
    const __nv_bfloat16* WT[3];   // [out][in]
    const float* b[3];
    float* out;                   // rows x d_out
};

__device__ __forceinline__ int mf_round16(int n) { return (n + 15) & ~15; }

// stage K chunk k0 of layer l: B rows [0, nrows_pad) of WT (rows >= n are
// zero), and for layer 1 the A rows of the CTA's x tile
__device__ __forceinline__ void mf_stage(const MlpArgs& a, int l, int m0, int k0, unsigned char* buf)
{
    const int K = l == 0 ? a.d_in : a.H;
    const int n = l == 2 ? a.d_out : a.H;
    const int npad = mf_round16(n);
    const __nv_bfloat16* W = l == 0 ? a.WT[0] : l == 1 ? a.WT[1] : a.WT[2];  // no runtime index into the parameters
    unsigned char* sA = buf;
    unsigned char* sB = buf + TC_M * TC_BK * 2;
    const int nqa = l == 0 ? TC_M * (TC_BK / 8) : 0;
    const int nq = nqa + npad * (TC_BK / 8);
    for (int q0 = threadIdx.x; q0 < nq; q0 += 4 * TC_THREADS) {
        uint32_t w[4][4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = q0 + u * TC_THREADS;
            w[u][0] = w[u][1] = w[u][2] = w[u][3] = 0u;
            if (q >= nq) continue;
            const bool isA = q < nqa;
            const int qq = isA ? q : q - nqa;
            const int r = qq >> 3, kc = qq & 7;
            const int k = k0 + kc * 8;
            const int row = isA ? m0 + r : r;
            const bool in = isA ? row < a.rows : row < n;
            const int kvalid = in ? min(8, K - k) : 0;
            if (kvalid <= 0) continue;
            if (isA)
                tc_chunk(a.x, 1, (long long)row * a.d_in + k, 1, kvalid, w[u]);
            else
                tc_chunk(W, 1, (long long)row * K + k, 1, kvalid, w[u]);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int q = q0 + u * TC_THREADS;
            if (q >= nq) continue;
            const bool isA = q < nqa;
            const int qq = isA ? q : q - nqa;
            const int r = qq >> 3, kc = qq & 7;
            unsigned char* dst = isA ? sA + tc_off(TC_M, r, kc * 8) : sB + tc_off(npad, r, kc * 8);
            *(uint4*)dst = make_uint4(w[u][0], w[u][1], w[u][2], w[u][3]);
        }
    }
}

__global__ void __launch_bounds__(TC_THREADS) k_mlp_fwd(MlpArgs a, long long timeout_ns)
{
    extern __shared__ __align__(1024) unsigned char msm[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tmem_base;
    unsigned char* hbuf = msm + 2 * MF_BUF;
    const int m0 = blockIdx.x * TC_M;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = tmem_base;
    bool ok = true;
    int g = 0;  // K chunks issued so far (all layers): buffer g & 1
    const int row = m0 + warp * 32 + lane;
    for (int l = 0; l < 3 && ok; ++l) {
        const int K = l == 0 ? a.d_in : a.H;
        const int n = l == 2 ? a.d_out : a.H;
        const int npad = mf_round16(n);
        const uint32_t idesc = tc_idesc(TC_M, npad);
        const uint32_t acc_col = l == 1 ? 256u : 0u;
        const int nk = (K + TC_BK - 1) / TC_BK;
        for (int kt = 0; kt < nk && ok; ++kt, ++g) {
            const int b = g & 1;
            unsigned char* buf = msm + (size_t)b * MF_BUF;
            if (g >= 2) ok = mbar_wait(&bar[b], (uint32_t)(((g - 2) >> 1) & 1), timeout_ns);
            if (!__syncthreads_and(ok)) {
                ok = false;
                break;
            }
            mf_stage(a, l, m0, kt * TC_BK, buf);
            fence_proxy_async_smem();
            __syncthreads();
            if (threadIdx.x == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t b0 = smem_addr(buf + TC_M * TC_BK * 2);
                // layer 1: A from the staged chunk; layers 2 and 3: from H
                const uint32_t a0 = l == 0 ? smem_addr(buf) : smem_addr(hbuf) + (uint32_t)(kt * 4) * (TC_M * 32);
#pragma unroll
                for (int ks = 0; ks < TC_BK / 16; ++ks) {
                    if (kt * TC_BK + ks * 16 >= mf_round16(K)) break;
                    const uint64_t ad = tc_desc(a0 + ks * TC_M * 32, 128, 256);
                    const uint64_t bd = tc_desc(b0 + ks * npad * 32, 128, 256);
                    const uint32_t accf = (kt > 0 || ks > 0) ? 1u : 0u;
                    asm volatile(
                        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(taddr + acc_col),
                        "l"(ad), "l"(bd), "r"(idesc), "r"(accf)
                        : "memory");
                }
                asm volatile(
                    "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                        smem_addr(&bar[b]))
                    : "memory");
            }
        }
        if (!ok) break;
        // the layer's last commit covers every MMA issued before it
        ok = mbar_wait(&bar[(g - 1) & 1], (uint32_t)(((g - 1) >> 1) & 1), timeout_ns);
        ok = __syncthreads_and(ok) != 0;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (!ok) break;
        // epilogue: 16 accumulator columns at a time
        for (int c0 = 0; c0 < n; c0 += 16) {
            uint32_t r[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr + acc_col + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const float* bias = l == 0 ? a.b[0] : l == 1 ? a.b[1] : a.b[2];
            float bv[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) bv[j] = (c0 + j < n) ? __ldg(bias + c0 + j) : 0.f;
            if (l < 2) {
                // ReLU, BF16, into H at (row - m0, k = c0 + j); columns >= n
                // (up to the 16-aligned K of the next layer) hold zeros
                uint32_t pk[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const float v0 = (c0 + 2 * j < n) ? fmaxf(__uint_as_float(r[2 * j]) + bv[2 * j], 0.f) : 0.f;
                    const float v1 =
                        (c0 + 2 * j + 1 < n) ? fmaxf(__uint_as_float(r[2 * j + 1]) + bv[2 * j + 1], 0.f) : 0.f;
                    pk[j] = pack_bf16(__float2bfloat16(v0), __float2bfloat16(v1));
                }
                const int rl = warp * 32 + lane;
                *(uint4*)(hbuf + tc_off(TC_M, rl, c0)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                *(uint4*)(hbuf + tc_off(TC_M, rl, c0 + 8)) = make_uint4(pk[4], pk[5], pk[6], pk[7]);
            } else if (row < a.rows) {
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (c0 + j < n) a.out[(long long)row * n + c0 + j] = __uint_as_float(r[j]) + bv[j];
            }
        }
        if (l < 2) {
            // H complete before the next layer's MMAs read it (async proxy);
            // this layer's accumulator reads are done
            fence_proxy_async_smem();
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        }
    }
    if (!ok) {
        if (threadIdx.x == 0) atomicExch(&g_tc_err, 1);
        // g K chunks were committed (a chunk counts once its MMAs are
        // issued): one more bounded wait on the last commit before the
        // tensor memory is freed
        if (g > 0) mbar_wait(&bar[(g - 1) & 1], (uint32_t)(((g - 1) >> 1) & 1), timeout_ns);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(512) : "memory");
}

// GEMM path: 1 (default) the tcgen05 kernel and the fused inference pass,
// 2 the tcgen05 kernel per layer, 0 the warp-level mma.sync kernel
int g_gemm_path = 1;

cudaError_t gemm(const GemmArgs& g, cudaStream_t st)
{
    if (g.M <= 0 || g.N <= 0 || g.K <= 0) return cudaSuccess;
    if (g_gemm_path == 0) {
        dim3 grid((g.N + GT_N - 1) / GT_N, (g.M + GT_M - 1) / GT_M);
        k_gemm_bf16<<<grid, 128, 0, st>>>(g);
        return cudaGetLastError();
    }
    const long long tmo = 2000000000LL;  // 2 s
    // 64-column tiles when 128-column ones would leave most SMs idle
    const long long mt = (g.M + TC_M - 1) / TC_M;
    if (g.N <= 64 || mt * ((g.N + 127) / 128) < 152) {
        constexpr size_t smem = 2 * (size_t)(TC_M + 64) * TC_BK * 2;
        cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_gemm_tc<64><<<dim3((g.N + 63) / 64, (g.M + TC_M - 1) / TC_M), TC_THREADS, smem, st>>>(g, tmo);
    } else {
        constexpr size_t smem = 2 * (size_t)(TC_M + 128) * TC_BK * 2;
        cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_gemm_tc<128><<<dim3((g.N + 127) / 128, (g.M + TC_M - 1) / TC_M), TC_THREADS, smem, st>>>(g, tmo);
    }
    return cudaGetLastError();
}

// dY := dY * (Y > 0)  (ReLU backward, in place on the FP32 gradient)
__global__ void k_relu_back(long long n, const float* __restrict__ y, float* __restrict__ dy)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        if (!(y[i] > 0.f)) dy[i] = 0.f;
}

// column sums: db[j] = sum_i dY[i][j]  (one thread per column, fixed order)
__global__ void k_colsum(int M, int N, const float* __restrict__ dy, float* __restrict__ db)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    float s = 0.f;
    for (int i = 0; i < M; ++i) s += dy[(long long)i * N + j];
    db[j] = s;
}

// mean-squared-error gradient: d = (pred - target) * 2 / (M * n_out); loss partial sums
__global__ void k_mse(long long n, float scale, const float* __restrict__ pred, const float* __restrict__ tgt,
                      float* __restrict__ d, double* __restrict__ loss)
{
    __shared__ double red[34];
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float e = pred[i] - tgt[i];
        d[i] = 2.f * scale * e;
        s += (double)e * e;
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0) atomicAdd(loss, s * scale);
}

__global__ void k_adam(long long n, float lr, float b1, float b2, float eps, float c1, float c2,
                       float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, __nv_bfloat16* __restrict__ wbf)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        if (wbf) wbf[i] = __float2bfloat16(wi);
    }
}

__global__ void k_to_bf16(long long n, const float* __restrict__ a, __nv_bfloat16* __restrict__ b)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16(a[i]);
}

// wt[o][i] = w[i][o] (BF16, rows x cols -> cols x rows)
__global__ void k_transpose_bf16(int rows, int cols, const __nv_bfloat16* __restrict__ w,
                                 __nv_bfloat16* __restrict__ wt)
{
    const long long n = (long long)rows * cols;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int o = (int)(t / rows), i = (int)(t - (long long)o * rows);
        wt[t] = w[(long long)i * cols + o];
    }
}

int g1d(long long n) { return (int)std::min<long long>((n + 255) / 256, 4096); }

}  // namespace

// ------------------------------------------------------------------ model
struct sem_learner {
    int d_in = 0, H = 0, d_out = 0;
    // parameters: FP32 master, BF16 copies for the GEMMs, Adam moments, gradients
    float *W[3] = {}, *b[3] = {}, *gW[3] = {}, *gb[3] = {}, *mW[3] = {}, *vW[3] = {}, *mb[3] = {}, *vb[3] = {};
    __nv_bfloat16* Wbf[3] = {};
    // transposed BF16 copies [out][in] for the forward GEMMs (their K runs
    // contiguous, so the tensor-core operand staging uses vector loads);
    // rebuilt before a forward pass whenever the weights changed
    __nv_bfloat16* WbfT[3] = {};
    bool wt_dirty = true;
    int rows_cap = 0;
    float *h1 = nullptr, *h2 = nullptr, *out = nullptr, *d2 = nullptr, *d1 = nullptr, *dout = nullptr;
    __nv_bfloat16 *h1bf = nullptr, *h2bf = nullptr;
    double* loss = nullptr;
    long long adam_t = 0;
    long long forward_launches = 0;  // kernels launched by forward passes
    cudaStream_t stream = nullptr;
    std::string err;
    int din(int l) const { return l == 0 ? d_in : H; }
    int dout_(int l) const { return l == 2 ? d_out : H; }
};

static int lfail(sem_learner* L, int code, const std::string& m)
{
    if (L) L->err = m;
    return ctx_fail(code, m.c_str());
}

#define LCUDA(call)                                                                                  \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return lfail(L, SEM_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

static int ensure_rows(sem_learner* L, int rows)
{
    if (rows <= L->rows_cap) return SEM_OK;
    float** fb[] = {&L->h1, &L->h2, &L->out, &L->d2, &L->d1, &L->dout};
    for (float** p : fb)
        if (*p) cudaFree(*p);
    if (L->h1bf) cudaFree(L->h1bf);
    if (L->h2bf) cudaFree(L->h2bf);
    const size_t r = (size_t)rows;
    LCUDA(cudaMalloc(&L->h1, r * L->H * 4));
    LCUDA(cudaMalloc(&L->h2, r * L->H * 4));
    LCUDA(cudaMalloc(&L->d1, r * L->H * 4));
    LCUDA(cudaMalloc(&L->d2, r * L->H * 4));
    LCUDA(cudaMalloc(&L->out, r * L->d_out * 4));
    LCUDA(cudaMalloc(&L->dout, r * L->d_out * 4));
    LCUDA(cudaMalloc(&L->h1bf, r * L->H * 2));
    LCUDA(cudaMalloc(&L->h2bf, r * L->H * 2));
    L->rows_cap = rows;
    return SEM_OK;
}

extern "C" int sem_learner_create(sem_learner** out, int d_in, int hidden, int d_out, unsigned long long seed)
{
    if (!out || d_in <= 0 || hidden <= 0 || d_out <= 0) return ctx_fail(SEM_ERR_ARG, "bad learner shape");
    sem_learner* L = new sem_learner();
    L->d_in = d_in;
    L->H = hidden;
    L->d_out = d_out;
    LCUDA(cudaMalloc(&L->loss, sizeof(double)));
    // He-uniform initialisation from a splitmix64 stream (host), biases zero
    uint64_t s = seed ? seed : 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < 3; ++l) {
        const size_t nw = (size_t)L->din(l) * L->dout_(l), nb = (size_t)L->dout_(l);
        std::vector<float> w(nw), z(nw > nb ? nw : nb, 0.f);
        const double a = std::sqrt(6.0 / L->din(l)) * (l == 2 ? 0.1 : 1.0);
        for (auto& v : w) v = (float)((2.0 * next() - 1.0) * a);
        float** bufs[] = {&L->W[l], &L->gW[l], &L->mW[l], &L->vW[l]};
        for (float** p : bufs) LCUDA(cudaMalloc(p, nw * 4));
        float** bb[] = {&L->b[l], &L->gb[l], &L->mb[l], &L->vb[l]};
        for (float** p : bb) LCUDA(cudaMalloc(p, nb * 4));
        LCUDA(cudaMalloc(&L->Wbf[l], nw * 2));
        LCUDA(cudaMalloc(&L->WbfT[l], nw * 2));
        LCUDA(cudaMemcpy(L->W[l], w.data(), nw * 4, cudaMemcpyHostToDevice));
        LCUDA(cudaMemset(L->mW[l], 0, nw * 4));
        LCUDA(cudaMemset(L->vW[l], 0, nw * 4));
        LCUDA(cudaMemset(L->b[l], 0, nb * 4));
        LCUDA(cudaMemset(L->mb[l], 0, nb * 4));
        LCUDA(cudaMemset(L->vb[l], 0, nb * 4));
        k_to_bf16<<<g1d(nw), 256>>>(nw, L->W[l], L->Wbf[l]);
        LCUDA(cudaGetLastError());
    }
    LCUDA(cudaDeviceSynchronize());
    *out = L;
    return SEM_OK;
}

extern "C" int sem_learner_destroy(sem_learner* L)
{
    if (!L) return SEM_OK;
    cudaDeviceSynchronize();
    for (int l = 0; l < 3; ++l) {
        float* f[] = {L->W[l], L->b[l], L->gW[l], L->gb[l], L->mW[l], L->vW[l], L->mb[l], L->vb[l]};
        for (float* p : f)
            if (p) cudaFree(p);
        if (L->Wbf[l]) cudaFree(L->Wbf[l]);
        if (L->WbfT[l]) cudaFree(L->WbfT[l]);
    }
    float* f2[] = {L->h1, L->h2, L->out, L->d2, L->d1, L->dout};
    for (float* p : f2)
        if (p) cudaFree(p);
    if (L->h1bf) cudaFree(L->h1bf);
    if (L->h2bf) cudaFree(L->h2bf);
    if (L->loss) cudaFree(L->loss);
    delete L;
    return SEM_OK;
}

extern "C" int sem_learner_shape(const sem_learner* L, int* d_in, int* hidden, int* d_out)
{
    if (!L) return ctx_fail(SEM_ERR_ARG, "null learner");
    if (d_in) *d_in = L->d_in;
    if (hidden) *hidden = L->H;
    if (d_out) *d_out = L->d_out;
    return SEM_OK;
}

extern "C" int sem_learner_set_stream(sem_learner* L, void* stream)
{
    if (!L) return ctx_fail(SEM_ERR_ARG, "null learner");
    L->stream = (cudaStream_t)stream;
    return SEM_OK;
}

// host copies of the FP32 parameters of layer l (W: d_in(l) x d_out(l) row-major, b: d_out(l))
extern "C" int sem_learner_get_params(sem_learner* L, int l, float* W, float* b)
{
    if (!L || l < 0 || l > 2) return ctx_fail(SEM_ERR_ARG, "bad layer");
    LCUDA(cudaStreamSynchronize(L->stream));
    if (W) LCUDA(cudaMemcpy(W, L->W[l], (size_t)L->din(l) * L->dout_(l) * 4, cudaMemcpyDeviceToHost));
    if (b) LCUDA(cudaMemcpy(b, L->b[l], (size_t)L->dout_(l) * 4, cudaMemcpyDeviceToHost));
    return SEM_OK;
}

extern "C" int sem_learner_set_params(sem_learner* L, int l, const float* W, const float* b)
{
    if (!L || l < 0 || l > 2) return ctx_fail(SEM_ERR_ARG, "bad layer");
    const size_t nw = (size_t)L->din(l) * L->dout_(l);
    if (W) {
        LCUDA(cudaMemcpy(L->W[l], W, nw * 4, cudaMemcpyHostToDevice));
        k_to_bf16<<<g1d(nw), 256, 0, L->stream>>>(nw, L->W[l], L->Wbf[l]);
        L->wt_dirty = true;
        LCUDA(cudaGetLastError());
    }
    if (b) LCUDA(cudaMemcpy(L->b[l], b, (size_t)L->dout_(l) * 4, cudaMemcpyHostToDevice));
    LCUDA(cudaStreamSynchronize(L->stream));
    return SEM_OK;
}

// transposed BF16 weights [out][in] for the forward pass, rebuilt after an
// update
static int refresh_wt(sem_learner* L)
{
    if (!L->wt_dirty) return SEM_OK;
    for (int l = 0; l < 3; ++l) {
        const long long nw = (long long)L->din(l) * L->dout_(l);
        k_transpose_bf16<<<g1d(nw), 256, 0, L->stream>>>(L->din(l), L->dout_(l), L->Wbf[l], L->WbfT[l]);
    }
    LCUDA(cudaGetLastError());
    L->wt_dirty = false;
    L->forward_launches += 3;
    return SEM_OK;
}

// the fused inference pass applies (tcgen05 path, hidden and output widths
// within one accumulator each)
static bool fused_forward_ok(const sem_learner* L)
{
    return g_gemm_path == 1 && L->H <= 256 && L->d_out <= 256;
}

// inference: x (rows x d_in, BF16) -> out (rows x d_out, FP32) in one launch
static int forward_fused(sem_learner* L, int rows, const __nv_bfloat16* x, float* out)
{
    int s = refresh_wt(L);
    if (s) return s;
    MlpArgs a{};
    a.rows = rows;
    a.d_in = L->d_in;
    a.H = L->H;
    a.d_out = L->d_out;
    a.x = x;
    a.out = out;
    for (int l = 0; l < 3; ++l) {
        a.WT[l] = L->WbfT[l];
        a.b[l] = L->b[l];
    }
    LCUDA(cudaFuncSetAttribute(k_mlp_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MF_SMEM));
    k_mlp_fwd<<<(rows + TC_M - 1) / TC_M, TC_THREADS, MF_SMEM, L->stream>>>(a, 2000000000LL);
    LCUDA(cudaGetLastError());
    L->forward_launches += 1;
    return SEM_OK;
}

// x: rows x d_in (device, BF16) -> L->out (FP32, rows x d_out), keeping
// the hidden activations for the backward pass
static int forward(sem_learner* L, int rows, const __nv_bfloat16* x)
{
    int s = ensure_rows(L, rows);
    if (s) return s;
    if ((s = refresh_wt(L))) return s;
    // B(k, n) = W[k][n] = WT[n][k]: K contiguous
    GemmArgs g{};
    g.M = rows; g.N = L->H; g.K = L->d_in;
    g.A = x; g.sa_m = L->d_in; g.sa_k = 1; g.a_bf16 = 1;
    g.B = L->WbfT[0]; g.sb_k = 1; g.sb_n = L->d_in; g.b_bf16 = 1;
    g.C = L->h1; g.ldc = L->H; g.bias = L->b[0]; g.relu = 1; g.Cbf = L->h1bf;
    LCUDA(gemm(g, L->stream));
    g.K = L->H; g.A = L->h1bf; g.sa_m = L->H;
    g.B = L->WbfT[1]; g.sb_n = L->H; g.C = L->h2; g.bias = L->b[1]; g.Cbf = L->h2bf;
    LCUDA(gemm(g, L->stream));
    g.N = L->d_out; g.A = L->h2bf; g.B = L->WbfT[2]; g.sb_n = L->H;
    g.C = L->out; g.ldc = L->d_out; g.bias = L->b[2]; g.relu = 0; g.Cbf = nullptr;
    LCUDA(gemm(g, L->stream));
    L->forward_launches += 3;
    return SEM_OK;
}

long long learner_forward_launches(const sem_learner* L) { return L ? L->forward_launches : 0; }

// predictions for rows x d_in BF16 inputs into out (device FP32, rows x d_out)
extern "C" int sem_learner_forward(sem_learner* L, int rows, const void* x_bf16, float* out)
{
    if (!L || rows < 0 || !x_bf16 || !out) return ctx_fail(SEM_ERR_ARG, "bad forward arguments");
    if (rows == 0) return SEM_OK;
    if (fused_forward_ok(L)) return forward_fused(L, rows, (const __nv_bfloat16*)x_bf16, out);
    int s = forward(L, rows, (const __nv_bfloat16*)x_bf16);
    if (s) return s;
    LCUDA(cudaMemcpyAsync(out, L->out, (size_t)rows * L->d_out * 4, cudaMemcpyDeviceToDevice, L->stream));
    return SEM_OK;
}

// gradients of the mean-squared error for one batch (device inputs); loss
// (mean over rows and outputs) to *loss_out; with lr > 0 also one Adam step
extern "C" int sem_learner_train_step(sem_learner* L, int rows, const void* x_bf16, const float* target,
                                      float lr, double* loss_out)
{
    if (!L || rows <= 0 || !x_bf16 || !target) return ctx_fail(SEM_ERR_ARG, "bad train arguments");
    const __nv_bfloat16* x = (const __nv_bfloat16*)x_bf16;
    int s = forward(L, rows, x);
    if (s) return s;
    const long long no = (long long)rows * L->d_out;
    LCUDA(cudaMemsetAsync(L->loss, 0, sizeof(double), L->stream));
    k_mse<<<g1d(no), 256, 0, L->stream>>>(no, 1.f / (float)no, L->out, target, L->dout, L->loss);
    LCUDA(cudaGetLastError());
    // layer 3: gW3 = h2^T dout, gb3 = colsum(dout), d2 = dout W3^T (masked by ReLU)
    GemmArgs g{};
    g.M = L->H; g.N = L->d_out; g.K = rows;
    g.A = L->h2bf; g.sa_m = 1; g.sa_k = L->H; g.a_bf16 = 1;
    g.B = L->dout; g.sb_k = L->d_out; g.sb_n = 1; g.b_bf16 = 0;
    g.C = L->gW[2]; g.ldc = L->d_out;
    LCUDA(gemm(g, L->stream));
    k_colsum<<<(L->d_out + 127) / 128, 128, 0, L->stream>>>(rows, L->d_out, L->dout, L->gb[2]);
    g = GemmArgs{};
    g.M = rows; g.N = L->H; g.K = L->d_out;
    g.A = L->dout; g.sa_m = L->d_out; g.sa_k = 1; g.a_bf16 = 0;
    g.B = L->Wbf[2]; g.sb_k = 1; g.sb_n = L->d_out; g.b_bf16 = 1;
    g.C = L->d2; g.ldc = L->H;
    LCUDA(gemm(g, L->stream));
    k_relu_back<<<g1d((long long)rows * L->H), 256, 0, L->stream>>>((long long)rows * L->H, L->h2, L->d2);
    // layer 2
    g = GemmArgs{};
    g.M = L->H; g.N = L->H; g.K = rows;
    g.A = L->h1bf; g.sa_m = 1; g.sa_k = L->H; g.a_bf16 = 1;
    g.B = L->d2; g.sb_k = L->H; g.sb_n = 1; g.b_bf16 = 0;
    g.C = L->gW[1]; g.ldc = L->H;
    LCUDA(gemm(g, L->stream));
    k_colsum<<<(L->H + 127) / 128, 128, 0, L->stream>>>(rows, L->H, L->d2, L->gb[1]);
    g = GemmArgs{};
    g.M = rows; g.N = L->H; g.K = L->H;
    g.A = L->d2; g.sa_m = L->H; g.sa_k = 1; g.a_bf16 = 0;
    g.B = L->Wbf[1]; g.sb_k = 1; g.sb_n = L->H; g.b_bf16 = 1;
    g.C = L->d1; g.ldc = L->H;
    LCUDA(gemm(g, L->stream));
    k_relu_back<<<g1d((long long)rows * L->H), 256, 0, L->stream>>>((long long)rows * L->H, L->h1, L->d1);
    // layer 1
    g = GemmArgs{};
    g.M = L->d_in; g.N = L->H; g.K = rows;
    g.A = x; g.sa_m = 1; g.sa_k = L->d_in; g.a_bf16 = 1;
    g.B = L->d1; g.sb_k = L->H; g.sb_n = 1; g.b_bf16 = 0;
    g.C = L->gW[0]; g.ldc = L->H;
    LCUDA(gemm(g, L->stream));
    k_colsum<<<(L->H + 127) / 128, 128, 0, L->stream>>>(rows, L->H, L->d1, L->gb[0]);
    LCUDA(cudaGetLastError());
    if (lr > 0.f) {
        ++L->adam_t;
        L->wt_dirty = true;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.f - std::pow(b1, (float)L->adam_t), c2 = 1.f - std::pow(b2, (float)L->adam_t);
        for (int l = 0; l < 3; ++l) {
            const long long nw = (long long)L->din(l) * L->dout_(l), nb = L->dout_(l);
            k_adam<<<g1d(nw), 256, 0, L->stream>>>(nw, lr, b1, b2, 1e-8f, c1, c2, L->W[l], L->gW[l], L->mW[l],
                                                   L->vW[l], L->Wbf[l]);
            k_adam<<<g1d(nb), 256, 0, L->stream>>>(nb, lr, b1, b2, 1e-8f, c1, c2, L->b[l], L->gb[l], L->mb[l],
                                                   L->vb[l], nullptr);
        }
        LCUDA(cudaGetLastError());
    }
    if (loss_out) {
        LCUDA(cudaMemcpyAsync(loss_out, L->loss, sizeof(double), cudaMemcpyDeviceToHost, L->stream));
        LCUDA(cudaStreamSynchronize(L->stream));
    }
    return SEM_OK;
}

// host copies of the last train step's gradients of layer l
extern "C" int sem_learner_get_grads(sem_learner* L, int l, float* gW, float* gb)
{
    if (!L || l < 0 || l > 2) return ctx_fail(SEM_ERR_ARG, "bad layer");
    LCUDA(cudaStreamSynchronize(L->stream));
    if (gW) LCUDA(cudaMemcpy(gW, L->gW[l], (size_t)L->din(l) * L->dout_(l) * 4, cudaMemcpyDeviceToHost));
    if (gb) LCUDA(cudaMemcpy(gb, L->gb[l], (size_t)L->dout_(l) * 4, cudaMemcpyDeviceToHost));
    return SEM_OK;
}

namespace {
__global__ void k_gather_rows(int rows, int dx, int dt, const int* __restrict__ idx,
                              const __nv_bfloat16* __restrict__ X, const float* __restrict__ T,
                              __nv_bfloat16* __restrict__ Xb, float* __restrict__ Tb)
{
    const long long total_x = (long long)rows * dx, total_t = (long long)rows * dt;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total_x; i += (long long)gridDim.x * blockDim.x)
        Xb[i] = X[(long long)idx[i / dx] * dx + i % dx];
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total_t; i += (long long)gridDim.x * blockDim.x)
        Tb[i] = T[(long long)idx[i / dt] * dt + i % dt];
}
}  // namespace

// Adam on the mean-squared error over a dataset of `rows` (BF16 inputs X,
// FP32 targets T, device), in shuffled minibatches; mean loss of the last
// epoch to *final_loss.
extern "C" int sem_learner_fit(sem_learner* L, const void* X, const float* T, long long rows, int epochs,
                               int batch, float lr, unsigned long long seed, double* final_loss)
{
    if (!L || !X || !T || rows <= 0 || epochs <= 0 || batch <= 0) return ctx_fail(SEM_ERR_ARG, "bad fit arguments");
    const int dx = L->d_in, dt = L->d_out;
    const int B = (int)std::min<long long>(batch, rows);
    int* didx = nullptr;
    __nv_bfloat16* Xb = nullptr;
    float* Tb = nullptr;
    LCUDA(cudaMalloc(&didx, sizeof(int) * B));
    LCUDA(cudaMalloc(&Xb, sizeof(__nv_bfloat16) * (size_t)B * dx));
    LCUDA(cudaMalloc(&Tb, sizeof(float) * (size_t)B * dt));
    std::vector<int> perm((size_t)rows);
    for (long long i = 0; i < rows; ++i) perm[(size_t)i] = (int)i;
    uint64_t s = seed ? seed : 12345u;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    double last = 0.0;
    int status = SEM_OK;
    for (int ep = 0; ep < epochs && status == SEM_OK; ++ep) {
        for (long long i = rows - 1; i > 0; --i) std::swap(perm[(size_t)i], perm[(size_t)(next() % (uint64_t)(i + 1))]);
        double sum = 0.0;
        int nb = 0;
        for (long long b0 = 0; b0 + B <= rows; b0 += B) {
            cudaMemcpyAsync(didx, perm.data() + b0, sizeof(int) * B, cudaMemcpyHostToDevice, L->stream);
            k_gather_rows<<<g1d((long long)B * dx), 256, 0, L->stream>>>(B, dx, dt, didx, (const __nv_bfloat16*)X, T,
                                                                         Xb, Tb);
            double loss = 0.0;
            status = sem_learner_train_step(L, B, Xb, Tb, lr, &loss);
            if (status) break;
            if (!std::isfinite(loss)) {
                status = lfail(L, SEM_ERR_ARG, "non-finite training loss (inputs, targets or learning rate)");
                break;
            }
            sum += loss;
            ++nb;
        }
        last = nb ? sum / nb : 0.0;
    }
    cudaFree(didx);
    cudaFree(Xb);
    cudaFree(Tb);
    if (status) return status;
    if (final_loss) *final_loss = last;
    return SEM_OK;
}

extern "C" int sem_gemm_set_path(int path)
{
    if (path < 0 || path > 2)
        return ctx_fail(SEM_ERR_ARG, "gemm path must be 0 (mma.sync), 1 (tcgen05, fused inference) or 2 (tcgen05)");
    g_gemm_path = path;
    return SEM_OK;
}

extern "C" int sem_gemm_check_error(int* expired)
{
    if (!expired) return ctx_fail(SEM_ERR_ARG, "null argument");
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_tc_err, sizeof(int));
    if (e != cudaSuccess) return ctx_fail(SEM_ERR_CUDA, cudaGetErrorString(e));
    *expired = v;
    return SEM_OK;
}

// generic BF16 tensor-core GEMM exposed for testing: C(M x N, FP32, row-major)
// = A(M x K, BF16 row-major) * B(K x N, BF16 row-major)
extern "C" int sem_gemm_bf16(int M, int N, int K, const void* A, const void* B, float* C, void* stream)
{
    if (M < 0 || N < 0 || K < 0 || (M && N && K && (!A || !B || !C))) return ctx_fail(SEM_ERR_ARG, "bad gemm");
    GemmArgs g{};
    g.M = M; g.N = N; g.K = K;
    g.A = A; g.sa_m = K; g.sa_k = 1; g.a_bf16 = 1;
    g.B = B; g.sb_k = N; g.sb_n = 1; g.b_bf16 = 1;
    g.C = C; g.ldc = N;
    cudaError_t e = gemm(g, (cudaStream_t)stream);
    if (e != cudaSuccess) return ctx_fail(SEM_ERR_CUDA, cudaGetErrorString(e));
    return SEM_OK;
}
