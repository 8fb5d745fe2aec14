// On-chip resident FP32 inner MINRES for the Schroedinger stage operator with
// the element fast-diagonalisation preconditioner, inside the same FP64
// iterative refinement as k_minres_mixed.
//
// When a block's share of the mesh fits in shared memory and registers (up to
// RES_TPB * RES_NPT element-local nodes, e.g. 31 elements at p = 8), every
// vector of the inner Krylov iteration stays on chip for the whole solve:
// r_{i-1}, r_i, z_i, the element operator output and the preconditioner's
// staging in shared memory, and the solution correction, the two direction
// vectors and z_{i-1} in registers of the thread that owns the node.  Only the
// element-ring copies (sides and corners, 4(N-1) of N^2 nodes) leave the SM:
// each is published as a 64-bit word (FP32 value, epoch tag) and the
// neighbours assemble every shared node from those words in the library's
// fixed order (dss_value's sums), so every copy of a node holds the same
// bits.  Per iteration:
//   Phase B: y = DSS(A_local z_i)/beta_i - (beta_i/beta_{i-1}) r_{i-1};
//            alpha partial z_i.y / beta_i; element preconditioner solves of y
//            (ring words out)                        -> exchange (alpha)
//   Phase A: z_{i+1} = DSS(local solves) - (alpha_i/beta_i) z_i;
//            y5 = y - (alpha_i/beta_i) r_i; beta_{i+1}^2 partial y5.z_{i+1};
//            element operator of z_{i+1} (ring words out) -> exchange (beta)
//   Givens rotation and the x / w update, in registers
// which is the iteration of minres_core<N, float, OP_RES, 2> (Paige-Saunders
// MINRES, include/minres.hpp:19-107 with a preconditioner).  An exchange is
// a grid all-reduce and the ring assembly at once (res_exchange).

// Differences from the staged kernel, all at the FP32 inner solve's rounding
// level: the right-hand side is scaled to unit norm (the correction is scaled
// back into the FP64 solution), the scalar recurrences run in FP32 on every
// thread (no broadcast, no FP64 pipe on the critical path), and block partial
// sums enter the grid sum as FP32.  The FP64 refinement judges the true
// residual exactly as k_minres_mixed does.
//
// Element contractions are line based: one thread takes one element line
// (N values in registers) and produces the N results of a 1-D contraction
// with the D or S coefficients as kernel-parameter (constant bank) operands,
// so a pass reads and writes each value once in shared memory.
//
// All-reduce: each block publishes its partial as one 64-bit word (FP32
// value, 32-bit epoch tag, each word on its own 128-byte line); every block's
// first warp polls the grid's words (bounded by SEM_OPT_WAIT_TIMEOUT_MS
// through %globaltimer) and sums them in one fixed order, so every block
// obtains the same bits.  Two word sets alternate by epoch parity; the host
// clears them, and the ring words, before each launch.
#pragma once
#include "sem_solvers.cuh"

namespace semgb {

constexpr int RES_TPB = 512;
constexpr int RES_NPT = 5;      // element-local nodes per thread (registers)
constexpr int RES_MAXQ = 8;     // words polled per lane: grids up to 256 blocks
constexpr int RES_PLANES = 18;  // FP32 planes of st values in shared memory
constexpr int RES_WSTRIDE = RESIDENT_SLOT_STRIDE;  // all-reduce words 128 bytes apart

// D(i,k) at [i*N+k] and the preconditioner basis S(i,k) at [i*N+k], passed
// by value: the unrolled contractions read them as constant-bank operands
template <int N>
struct ResCoef {
    float D[N * N];
    float S[N * N];
};

struct ResArgs {
    int st;                     // shared-memory plane length (max elements per block * N^2)
    unsigned long long* xa;     // [2 n] tagged ring words of the operator output, zero at launch
    unsigned long long* xb;     // [2 n] tagged ring words of the preconditioner output, zero at launch
    unsigned long long* slots;  // [2][gridDim.x][RES_WSTRIDE] tagged partial sums, zero at launch
};

// one 64-bit word: FP32 value in the low half, epoch in the high half
__device__ __forceinline__ unsigned long long res_word(float v, unsigned epoch)
{
    return ((unsigned long long)epoch << 32) | (unsigned long long)__float_as_uint(v);
}

__device__ __forceinline__ unsigned long long res_ld(const unsigned long long* p)
{
    return *(const volatile unsigned long long*)p;
}

// ---------------------------------------------------------------- line passes
// xi lines (c, le, j): N consecutive values from base = c*st + le*N^2 + j*N;
// eta lines (c, le, i): stride N from base = c*st + le*N^2 + i.  Line L is
// (c, pos, le) with the element fastest.  Lines of one pass are disjoint, so
// each pass may write in place.
// element count of the block and its FP32 reciprocal: (rem + 0.5) * (1/ne)
// in FP32 is at least 0.5 / ne from an integer and within a few ulp of the
// exact quotient, so its truncation is rem / ne (checked exhaustively for
// ne <= 1024, rem < 34 ne)
struct ResNe {
    int n;
    float inv;
};
template <int N>
__device__ __forceinline__ void res_line(int L, ResNe ne, int st, bool xi, int& base, int& fb, int& pos)
{
    constexpr int NN = N * N;
    const int per = ne.n * N;
    const int c = L >= per ? 1 : 0;
    const int rem = L - c * per;
    pos = (int)(((float)rem + 0.5f) * ne.inv);  // rem / ne: j of a xi line, i of an eta line
    // consecutive threads take the same line of consecutive elements: with an
    // odd N the element stride N^2 spreads a warp over all 32 banks
    const int le = rem - pos * ne.n;
    fb = le * NN + (xi ? pos * N : pos);
    base = c * st + fb;
}

// apply pass X1: A = D u along xi (u_xi)
template <int N>
__device__ __forceinline__ void res_apply_x1(const ResCoef<N>& cf, const float* U, float* A, ResNe ne, int st)
{
    for (int L = threadIdx.x; L < 2 * ne.n * N; L += RES_TPB) {
        int base, fb, pos;
        res_line<N>(L, ne, st, true, base, fb, pos);
        float u[N];
#pragma unroll
        for (int k = 0; k < N; ++k) u[k] = U[base + k];
#pragma unroll
        for (int i = 0; i < N; ++i) {
            float a = 0.f;
#pragma unroll
            for (int k = 0; k < N; ++k) a = fmaf(cf.D[i * N + k], u[k], a);
            A[base + i] = a;
        }
    }
}

// apply pass Y1: u_eta along eta, then the contravariant fluxes
// f1 = g11 u_xi - g12 u_eta (into A) and f2 = g22 u_eta - g12 u_xi (into B)
template <int N>
__device__ __forceinline__ void res_apply_y1(const ResCoef<N>& cf, const float* U, float* A, float* B,
                                             const float* G11, const float* G12, const float* G22, ResNe ne, int st)
{
    for (int L = threadIdx.x; L < 2 * ne.n * N; L += RES_TPB) {
        int base, fb, pos;
        res_line<N>(L, ne, st, false, base, fb, pos);
        float u[N], ur[N];
#pragma unroll
        for (int k = 0; k < N; ++k) {
            u[k] = U[base + k * N];
            ur[k] = A[base + k * N];
        }
#pragma unroll
        for (int j = 0; j < N; ++j) {
            float us = 0.f;
#pragma unroll
            for (int k = 0; k < N; ++k) us = fmaf(cf.D[j * N + k], u[k], us);
            const float g11 = G11[fb + j * N], g12 = G12[fb + j * N], g22 = G22[fb + j * N];
            A[base + j * N] = g11 * ur[j] - g12 * us;
            B[base + j * N] = g22 * us - g12 * ur[j];
        }
    }
}

// apply pass X2: A = D^T f1 along xi (first half of the weak divergence)
template <int N>
__device__ __forceinline__ void res_apply_x2(const ResCoef<N>& cf, float* A, ResNe ne, int st)
{
    for (int L = threadIdx.x; L < 2 * ne.n * N; L += RES_TPB) {
        int base, fb, pos;
        res_line<N>(L, ne, st, true, base, fb, pos);
        float f[N];
#pragma unroll
        for (int k = 0; k < N; ++k) f[k] = A[base + k];
#pragma unroll
        for (int i = 0; i < N; ++i) {
            float a = 0.f;
#pragma unroll
            for (int k = 0; k < N; ++k) a = fmaf(cf.D[k * N + i], f[k], a);
            A[base + i] = a;
        }
    }
}

// apply pass Y2: A += D^T f2 along eta (continuing the same FMA chain)
template <int N>
__device__ __forceinline__ void res_apply_y2(const ResCoef<N>& cf, float* A, const float* B, ResNe ne, int st)
{
    for (int L = threadIdx.x; L < 2 * ne.n * N; L += RES_TPB) {
        int base, fb, pos;
        res_line<N>(L, ne, st, false, base, fb, pos);
        float f[N], a1[N];
#pragma unroll
        for (int k = 0; k < N; ++k) {
            f[k] = B[base + k * N];
            a1[k] = A[base + k * N];
        }
#pragma unroll
        for (int j = 0; j < N; ++j) {
            float a = a1[j];
#pragma unroll
            for (int k = 0; k < N; ++k) a = fmaf(cf.D[k * N + j], f[k], a);
            A[base + j * N] = a;
        }
    }
}

// preconditioner passes on B in place (fdm_range_post's four contractions):
// F1 t = S^T u along xi; F2 u = d * (t S) along eta; F3 t = S u along xi;
// F4 z = t S^T along eta, times the Neumann-Neumann weight, ring copies to Xout
// (tagged words, see res_exchange)
template <int N>
__device__ __forceinline__ void res_fdm_xi(const ResCoef<N>& cf, float* B, ResNe ne, int st, bool transpose)
{
    for (int L = threadIdx.x; L < 2 * ne.n * N; L += RES_TPB) {
        int base, fb, pos;
        res_line<N>(L, ne, st, true, base, fb, pos);
        float u[N];
#pragma unroll
        for (int k = 0; k < N; ++k) u[k] = B[base + k];
#pragma unroll
        for (int a = 0; a < N; ++a) {
            float acc = 0.f;
#pragma unroll
            for (int i = 0; i < N; ++i) acc = fmaf(transpose ? cf.S[i * N + a] : cf.S[a * N + i], u[i], acc);
            B[base + a] = acc;
        }
    }
}

template <int N>
__device__ __forceinline__ void res_fdm_f2(const ResCoef<N>& cf, float* B, const float* FD, ResNe ne, int st)
{
    for (int L = threadIdx.x; L < 2 * ne.n * N; L += RES_TPB) {
        int base, fb, pos;
        res_line<N>(L, ne, st, false, base, fb, pos);
        float t[N];
#pragma unroll
        for (int k = 0; k < N; ++k) t[k] = B[base + k * N];
#pragma unroll
        for (int b = 0; b < N; ++b) {
            float acc = 0.f;
#pragma unroll
            for (int j = 0; j < N; ++j) acc = fmaf(t[j], cf.S[j * N + b], acc);
            B[base + b * N] = FD[fb + b * N] * acc;
        }
    }
}

template <int N>
__device__ __forceinline__ void res_fdm_f4(const ResCoef<N>& cf, float* B, const float* WT, unsigned long long* Xout,
                                           unsigned tag, ResNe ne, int st, long long n, int eb)
{
    constexpr int NN = N * N;
    for (int L = threadIdx.x; L < 2 * ne.n * N; L += RES_TPB) {
        int base, fb, pos;
        res_line<N>(L, ne, st, false, base, fb, pos);
        const int c = base >= st ? 1 : 0;
        const int le = fb / NN;
        const long long gbase = (long long)c * n + (long long)(eb + le) * NN + pos;  // node (pos, j)
        float t[N];
#pragma unroll
        for (int k = 0; k < N; ++k) t[k] = B[base + k * N];
        const bool side_i = (pos == 0) | (pos == N - 1);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            float acc = 0.f;
#pragma unroll
            for (int b = 0; b < N; ++b) acc = fmaf(t[b], cf.S[j * N + b], acc);
            const float z = WT[fb + j * N] * acc;
            B[base + j * N] = z;
            if (side_i || j == 0 || j == N - 1) __stcg(Xout + gbase + (long long)j * N, res_word(z, tag));
        }
    }
}

// ------------------------------------------------------- shared-memory planes
// plane p starts at p*st floats:
//   0 G11, 1 G12, 2 G22, 3 mass, 4 mass*V, 5 preconditioner diagonal,
//   6 Neumann-Neumann weight, 7 owner (1/0)           (constant per launch)
//   8-9 U (z_i, apply input), 10-11 A (operator output / apply scratch),
//   12-13 B (flux f2 / preconditioner staging), 14-15 R1, 16-17 R2
// The FP64 refinement's staging area overlays planes 8-17 between inner solves.
template <int N>
__device__ __forceinline__ void res_setup(const DevMesh& m, float* sm, int st, int eb, int ne, const float* pot32,
                                          float alpha)
{
    constexpr int NN = N * N;
    const float* lam = m.fdmL32;
    for (int l = threadIdx.x; l < ne * NN; l += RES_TPB) {
        const int le = l / NN;
        const int node = l - le * NN;
        const int i = node % N, j = node / N;
        const int e = eb + le;
        const long long flat = (long long)e * NN + node;
        const float ms = __ldg(m.massf + flat);
        sm[l] = __ldg(m.g11f + flat);
        sm[st + l] = __ldg(m.g12f + flat);
        sm[2 * st + l] = __ldg(m.g22f + flat);
        sm[3 * st + l] = ms;
        sm[4 * st + l] = ms * __ldg(pot32 + flat);
        const float4 g = __ldg(m.fdm_el + e);
        const float lk = g.y * __ldg(lam + i) + g.z * __ldg(lam + j);
        const float mm = g.x;
        sm[5 * st + l] = 1.f / sqrtf(mm * mm + alpha * alpha * lk * lk);
        const NodeInfo ni = node_info<N>(m, e, i, j);
        sm[6 * st + l] = nn_weight<N, float>(m, ni, e);
        sm[7 * st + l] = ni_owner(ni) ? 1.f : 0.f;
    }
}

// Assembly of the ring copies in place (continuous format, dss_value's
// sums), from tagged words.  The element-local planes P (two components) hold
// this block's partials; X holds every block's ring partials as 64-bit words
// (FP32 value, epoch tag `tag`), so a load that returns the right tag is the
// data itself: no flag, fence or barrier stands between a neighbour's store
// and its use.  One task per element side and component (its N-2 side
// nodes: own + the neighbour's copy at side_base + k side_step) and one per
// element corner and component (the corner node's copies in CSR order);
// stale words are reloaded until their tag matches (bounded: returns false
// after recording gs->err when tmo runs out).  Dirichlet boundary copies
// become zero; lone (Neumann) sides keep their own value.  Threads
// [t_first, RES_TPB) take the tasks.
template <int N>
__device__ __forceinline__ bool res_ring(const DevMesh& m, const unsigned long long* X, float* P, int st, int eb,
                                         int ne, unsigned tag, int t_first, GridSync* gs, long long tmo)
{
    constexpr int NN = N * N;
    const long long n = m.n;
    const int nside = ne * 8;  // (element, side, component)
    const int ntask = ne * 16;
    bool ok = true;
    const unsigned long long t0 = global_ns();
    for (int t = threadIdx.x - t_first; t < ntask && ok; t += RES_TPB - t_first) {
        const bool corner = t >= nside;
        const int u = corner ? t - nside : t;
        const int c = u & 1;
        const int sc = (u >> 1) & 3;
        const int le = u >> 3;
        const int e = eb + le;
        const int fl = __ldg(m.flags + e);
        float* pe = P + c * st + le * NN;
        const unsigned long long* x = X + (long long)c * n;
        if (!corner) {
            const int l0 = sc == 0 ? 0 : sc == 1 ? N - 1 : sc == 2 ? (N - 1) * N : 0;
            const int lk = (sc == 0 || sc == 2) ? 1 : N;
            if ((fl >> (4 + sc)) & 1) {  // Dirichlet boundary side
#pragma unroll
                for (int k = 1; k < N - 1; ++k) pe[l0 + k * lk] = 0.f;
            } else if (!((fl >> (16 + sc)) & 1)) {  // interior side: own + other
                const long long sb = __ldg(m.side_base + 4 * e + sc), ss = __ldg(m.side_step + 4 * e + sc);
                unsigned long long w[N];
#pragma unroll
                for (int k = 1; k < N - 1; ++k) w[k] = res_ld(x + sb + k * ss);
                for (unsigned polls = 1;; ++polls) {
                    bool ready = true;
#pragma unroll
                    for (int k = 1; k < N - 1; ++k) ready &= (unsigned)(w[k] >> 32) == tag;
                    if (ready) break;
                    if ((polls & 31u) == 0 &&
                        (*(volatile int*)&gs->err || (long long)(global_ns() - t0) > tmo)) {
                        atomicExch(&gs->err, 1);
                        ok = false;
                        break;
                    }
#pragma unroll
                    for (int k = 1; k < N - 1; ++k)
                        if ((unsigned)(w[k] >> 32) != tag) w[k] = res_ld(x + sb + k * ss);
                }
#pragma unroll
                for (int k = 1; k < N - 1; ++k)
                    pe[l0 + k * lk] = pe[l0 + k * lk] + __uint_as_float((unsigned)w[k]);
            }
        } else {
            const int lc = sc == 0 ? 0 : sc == 1 ? N - 1 : sc == 2 ? NN - 1 : (N - 1) * N;
            if ((fl >> (12 + sc)) & 1) {  // Dirichlet boundary corner
                pe[lc] = 0.f;
                continue;
            }
            const int* cl = m.corner_nb + (size_t)(4 * e + sc) * CORNER_NB_MAX;
            int q[CORNER_NB_MAX];
#pragma unroll
            for (int k = 0; k < CORNER_NB_MAX; ++k) q[k] = __ldg(cl + k);
            float sum = 0.f;  // csum = 0, then += in connected_elements order
            if (q[0] == -2) {  // more copies than the table holds: the CSR, one by one
                const int node = __ldg(m.corner_node + 4 * e + sc);
                const int q0 = __ldg(m.node_ptr + node), q1 = __ldg(m.node_ptr + node + 1);
                for (int k = q0; k < q1 && ok; ++k) {
                    const int f = __ldg(m.node_flat + k);
                    unsigned long long v = res_ld(x + f);
                    for (unsigned polls = 1; (unsigned)(v >> 32) != tag; ++polls) {
                        if ((polls & 31u) == 0 &&
                            (*(volatile int*)&gs->err || (long long)(global_ns() - t0) > tmo)) {
                            atomicExch(&gs->err, 1);
                            ok = false;
                            break;
                        }
                        v = res_ld(x + f);
                    }
                    sum += __uint_as_float((unsigned)v);
                }
            } else {
                unsigned long long w[CORNER_NB_MAX];
#pragma unroll
                for (int k = 0; k < CORNER_NB_MAX; ++k) w[k] = q[k] >= 0 ? res_ld(x + q[k]) : res_word(0.f, tag);
                for (unsigned polls = 1;; ++polls) {
                    bool ready = true;
#pragma unroll
                    for (int k = 0; k < CORNER_NB_MAX; ++k) ready &= (unsigned)(w[k] >> 32) == tag;
                    if (ready) break;
                    if ((polls & 31u) == 0 &&
                        (*(volatile int*)&gs->err || (long long)(global_ns() - t0) > tmo)) {
                        atomicExch(&gs->err, 1);
                        ok = false;
                        break;
                    }
#pragma unroll
                    for (int k = 0; k < CORNER_NB_MAX; ++k)
                        if ((unsigned)(w[k] >> 32) != tag) w[k] = res_ld(x + q[k]);
                }
#pragma unroll
                for (int k = 0; k < CORNER_NB_MAX; ++k)
                    if (q[k] >= 0) sum += __uint_as_float((unsigned)w[k]);
            }
            pe[lc] = sum;
        }
    }
    return ok;
}

// One phase boundary: the grid all-reduce of v (first warp: publish this
// block's word, poll every block's) and, at the same time, the in-place ring
// assembly of P from the tagged words X (the other warps).  Both wait for the
// same stores of the other blocks, so the phase costs one round trip after
// the last of them.  The ring words and the all-reduce word carry the same
// epoch.  Returns false when a wait hit its limit.
template <int N>
__device__ __forceinline__ bool res_exchange(float v, const DevMesh& m, const unsigned long long* X, float* P, int st,
                                             int eb, int ne, unsigned long long* slots, unsigned& epoch,
                                             GridSync* gs, long long tmo, double* red, double& out)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid] = (double)v;
    ++epoch;
    __syncthreads();
    bool ok = true;
    if (wid == 0) {
        constexpr int nw = RES_TPB / 32;
        double s = lane < nw ? red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        const int G = gridDim.x;
        unsigned long long* sl = slots + (size_t)(epoch & 1u) * G * RES_WSTRIDE;
        if (lane == 0) *(volatile unsigned long long*)(sl + blockIdx.x * RES_WSTRIDE) = res_word((float)s, epoch);
        unsigned long long u[RES_MAXQ];
#pragma unroll
        for (int k = 0; k < RES_MAXQ; ++k) {
            const int q = lane + 32 * k;
            u[k] = q < G ? res_ld(sl + q * RES_WSTRIDE) : res_word(0.f, epoch);
        }
        const unsigned long long t0 = global_ns();
        for (unsigned polls = 1;; ++polls) {
            bool ready = true;
#pragma unroll
            for (int k = 0; k < RES_MAXQ; ++k) ready &= (unsigned)(u[k] >> 32) == epoch;
            if (ready) break;
            if ((polls & 31u) == 0) {
                if (*(volatile int*)&gs->err || (long long)(global_ns() - t0) > tmo) {
                    atomicExch(&gs->err, 1);
                    ok = false;
                    break;
                }
            }
#pragma unroll
            for (int k = 0; k < RES_MAXQ; ++k) {
                const int q = lane + 32 * k;
                if (q < G && (unsigned)(u[k] >> 32) != epoch) u[k] = res_ld(sl + q * RES_WSTRIDE);
            }
        }
        double acc = 0.0;
#pragma unroll
        for (int k = 0; k < RES_MAXQ; ++k) acc += (double)__uint_as_float((unsigned)u[k]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) red[32] = acc;
    } else {
        ok = res_ring<N>(m, X, P, st, eb, ne, epoch, 32, gs, tmo);
    }
    const bool fail = __syncthreads_or(!ok) != 0;
    out = red[32];
    return !fail;
}

// Res combination on the line passes' laplacian (planes A), ring copies of
// the element-local result to the exchange words X (tag: the epoch of the
// exchange that reads them)
template <int N>
__device__ __forceinline__ void res_combine(const float* U, float* A, const float* MS, const float* MV,
                                            unsigned long long* X, unsigned tag, int st, int eb, int nl, float alpha,
                                            long long n)
{
    constexpr int NN = N * N;
#pragma unroll
    for (int k = 0; k < RES_NPT; ++k) {
        const int l = threadIdx.x + k * RES_TPB;
        if (l < nl) {
            const int le = l / NN, node = l - le * NN, i = node % N, j = node / N;
            const float u0 = U[l], u1 = U[st + l], ms = MS[l], mv = MV[l];
            const float Lv = A[st + l] + mv * u1;
            const float Lu = A[l] + mv * u0;
            const float o0 = ms * u0 + alpha * Lv;
            const float o1 = alpha * Lu - ms * u1;
            A[l] = o0;
            A[st + l] = o1;
            if ((i == 0) | (i == N - 1) | (j == 0) | (j == N - 1)) {
                const long long flat = (long long)(eb + le) * NN + node;
                __stcg(X + flat, res_word(o0, tag));
                __stcg(X + n + flat, res_word(o1, tag));
            }
        }
    }
}

template <int N>
__device__ __forceinline__ void res_apply(const ResCoef<N>& cf, float* sm, int st, int eb, int ne, float alpha,
                                          unsigned long long* X, unsigned tag, long long n)
{
    float* U = sm + 8 * st;
    float* A = sm + 10 * st;
    float* B = sm + 12 * st;
    const ResNe nb{ne, 1.f / (float)ne};
    __syncthreads();
    res_apply_x1<N>(cf, U, A, nb, st);
    __syncthreads();
    res_apply_y1<N>(cf, U, A, B, sm, sm + st, sm + 2 * st, nb, st);
    __syncthreads();
    res_apply_x2<N>(cf, A, nb, st);
    __syncthreads();
    res_apply_y2<N>(cf, A, B, nb, st);
    __syncthreads();
    res_combine<N>(U, A, sm + 3 * st, sm + 4 * st, X, tag, st, eb, ne * N * N, alpha, n);
}

template <int N>
__device__ __forceinline__ void res_precond(const ResCoef<N>& cf, float* sm, int st, int eb, int ne,
                                            unsigned long long* X, unsigned tag, long long n)
{
    float* B = sm + 12 * st;
    const ResNe nb{ne, 1.f / (float)ne};
    __syncthreads();
    res_fdm_xi<N>(cf, B, nb, st, true);
    __syncthreads();
    res_fdm_f2<N>(cf, B, sm + 5 * st, nb, st);
    __syncthreads();
    res_fdm_xi<N>(cf, B, nb, st, false);
    __syncthreads();
    res_fdm_f4<N>(cf, B, sm + 6 * st, X, tag, nb, st, n, eb);
}

struct ResOut {
    int it;
    bool conv;
};

// The inner solve A d = r (r: FP64 residual planes, continuous format, |r| = rn
// > 0) to relative tolerance tol_rel in the preconditioned norm, at most maxit
// iterations; adds d to the FP64 solution on owner copies.  Returns false
// when a wait hit its limit.
template <int N>
__device__ __forceinline__ bool res_inner(const DevMesh& m, const ResCoef<N>& cf, float* sm, int st, int eb, int ne,
                                          const double* const* r64, double rn, float alpha, unsigned long long* XA,
                                          unsigned long long* XB, unsigned long long* slots, unsigned& epoch,
                                          GridSync* gs, long long tmo,
                                          double* red, int maxit, float tol_rel, double* const* xp, ResOut& res)
{
    constexpr int NN = N * N;
    const long long n = m.n;
    const int nl = ne * NN;
    res.it = 0;
    res.conv = false;
    if (maxit < 1) return true;
    const float* WT = sm + 6 * st;
    const float* OW = sm + 7 * st;
    float* U = sm + 8 * st;
    float* A = sm + 10 * st;
    float* B = sm + 12 * st;
    float* Ra = sm + 14 * st;  // r_{i-1}, then y, then y5
    float* Rb = sm + 16 * st;  // r_i
    const float eps_mach = FLT_EPSILON;
    const double inv_rn = 1.0 / rn;
    const int t0 = threadIdx.x;
    // registers: solution correction, direction vectors, previous z
    float x[2][RES_NPT], w1[2][RES_NPT], w2[2][RES_NPT], zp[2][RES_NPT];
#pragma unroll
    for (int k = 0; k < RES_NPT; ++k)
#pragma unroll
        for (int c = 0; c < 2; ++c) x[c][k] = w1[c][k] = w2[c][k] = zp[c][k] = 0.f;

    // ---- P0: r_1 = r / |r|; preconditioner input wt * r; local solves
#pragma unroll
    for (int k = 0; k < RES_NPT; ++k) {
        const int l = t0 + k * RES_TPB;
        if (l < nl) {
            const long long flat = (long long)eb * NN + l;
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const float r = (float)(__ldcg(r64[c] + flat) * inv_rn);
                Rb[c * st + l] = r;
                B[c * st + l] = WT[l] * r;
            }
        }
    }
    res_precond<N>(cf, sm, st, eb, ne, XB, epoch + 1, n);
    double dummy = 0.0;
    if (!res_exchange<N>(0.f, m, XB, B, st, eb, ne, slots, epoch, gs, tmo, red, dummy)) return false;
    // ---- P1: z_1 = DSS(local solves) (assembled in B); |r|_P^2 = r.z; A = A_local(z_1)
    float pz = 0.f;
#pragma unroll
    for (int k = 0; k < RES_NPT; ++k) {
        const int l = t0 + k * RES_TPB;
        if (l < nl) {
            const float z0 = B[l], z1 = B[st + l];
            U[l] = z0;
            U[st + l] = z1;
            pz = fmaf(OW[l] * Rb[l], z0, pz);
            pz = fmaf(OW[l] * Rb[st + l], z1, pz);
        }
    }
    res_apply<N>(cf, sm, st, eb, ne, alpha, XA, epoch + 1, n);
    double bz = 0.0;
    if (!res_exchange<N>(pz, m, XA, A, st, eb, ne, slots, epoch, gs, tmo, red, bz)) return false;
    if (!(bz > 0.0)) {  // r . P^-1 r = 0: nothing to solve
        res.conv = true;
        return true;
    }
    // scalar state (minres.hpp:28-40; preconditioned norms)
    float beta = sqrtf((float)bz);
    float inv_beta = 1.f / beta;
    const float bnorm = beta;
    float phibar = beta, cs = -1.f, sn = 0.f, dbar = 0.f, eps = 0.f, c1 = 0.f;
    int it = 1;
    bool conv = false;
    for (;;) {
        // ---- Phase B_it (A holds the assembled A z_i)
        float s1 = 0.f;
#pragma unroll
        for (int k = 0; k < RES_NPT; ++k) {
            const int l = t0 + k * RES_TPB;
            if (l < nl) {
                const float av0 = A[l], av1 = A[st + l];
                const float ow = OW[l], wt = WT[l];
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const float a = (c == 0 ? av0 : av1) * inv_beta;
                    const float y = it >= 2 ? a - c1 * Ra[c * st + l] : a;
                    Ra[c * st + l] = y;
                    s1 = fmaf(ow * (inv_beta * U[c * st + l]), y, s1);
                    B[c * st + l] = wt * y;
                }
            }
        }
        res_precond<N>(cf, sm, st, eb, ne, XB, epoch + 1, n);
        double S1 = 0.0;
        if (!res_exchange<N>(s1, m, XB, B, st, eb, ne, slots, epoch, gs, tmo, red, S1)) return false;
        const float alpha_i = (float)S1;
        const float c2 = alpha_i * inv_beta;
        // ---- Phase A_it+1 (B holds the assembled local solves)
        float ss = 0.f;
#pragma unroll
        for (int k = 0; k < RES_NPT; ++k) {
            const int l = t0 + k * RES_TPB;
            if (l < nl) {
                const float q0 = B[l], q1 = B[st + l];
                const float ow = OW[l];
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const float zc = U[c * st + l];
                    zp[c][k] = zc;
                    const float zn = (c == 0 ? q0 : q1) - c2 * zc;
                    const float y5 = Ra[c * st + l] - c2 * Rb[c * st + l];
                    Ra[c * st + l] = y5;
                    U[c * st + l] = zn;
                    ss = fmaf(ow * y5, zn, ss);
                }
            }
        }
        res_apply<N>(cf, sm, st, eb, ne, alpha, XA, epoch + 1, n);
        double bnew2d = 0.0;
        if (!res_exchange<N>(ss, m, XA, A, st, eb, ne, slots, epoch, gs, tmo, red, bnew2d)) return false;
        {
            float* tmp = Ra;  // r_{i-1} <- r_i, r_i <- y5
            Ra = Rb;
            Rb = tmp;
        }
        // ---- Givens rotation of iteration it (minres.hpp:65-92), FP32
        const float bnew2 = bnew2d > 0.0 ? (float)bnew2d : 0.f;
        const float inv_beta_new = bnew2 > 0.f ? rsqrtf(bnew2) : 1.f / bnew2;
        const float beta_new = bnew2 > 0.f ? bnew2 * inv_beta_new : 0.f;
        const float eps_old = eps;
        const float delta = cs * dbar + sn * alpha_i;
        const float gbar = sn * dbar - cs * alpha_i;
        eps = sn * beta_new;
        dbar = -cs * beta_new;
        const float g2 = gbar * gbar + beta_new * beta_new;
        float ig = rsqrtf(g2), gamma = g2 * ig;
        if (!(gamma >= eps_mach)) {
            gamma = eps_mach;
            ig = 1.f / eps_mach;
        }
        cs = gbar * ig;
        sn = beta_new * ig;
        const float phi = cs * phibar;
        phibar *= sn;
        // w_it = (v_it - eps w_{it-2} - delta w_{it-1}) / gamma, x += phi w_it
        const float pinvb = inv_beta;
#pragma unroll
        for (int k = 0; k < RES_NPT; ++k)
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const float wn = ig * ((pinvb * zp[c][k] - eps_old * w1[c][k]) - delta * w2[c][k]);
                w1[c][k] = w2[c][k];
                w2[c][k] = wn;
                x[c][k] = fmaf(phi, wn, x[c][k]);
            }
        c1 = beta_new * inv_beta;
        beta = beta_new;
        inv_beta = inv_beta_new;
        conv = phibar < tol_rel * bnorm;  // minres.hpp:92 (relative part)
        if (conv || it == maxit || beta == 0.f) break;
        ++it;
    }
    // ---- x += d (FP64, owner copies): d = |r| * (the unit-rhs correction)
#pragma unroll
    for (int k = 0; k < RES_NPT; ++k) {
        const int l = t0 + k * RES_TPB;
        if (l < nl && OW[l] != 0.f) {
            const long long flat = (long long)eb * NN + l;
#pragma unroll
            for (int c = 0; c < 2; ++c) xp[c][flat] += (double)x[c][k] * rn;
        }
    }
    res.it = it;
    res.conv = conv;
    return true;
}

// ------------------------------------------------------------------ kernel
// FP64 iterative refinement (the sweep of mixed_solve: true residual
// r = b - A x, the reference's stopping test on |r|) around res_inner.
template <int N>
__global__ void __launch_bounds__(RES_TPB, 1)
    k_minres_resident(DevMesh m, SolveArgs a, KrylovWork<float> w, MixedArgs mx, ResCoef<N> cf, ResArgs ra)
{
    constexpr int NN = N * N;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[34];
    __shared__ double sweep_state[3];  // r0, |r|, done
    float* sm = (float*)smraw;
    const int st = ra.st;
    int eb, ee;
    block_range(m.E, eb, ee);
    const int ne = ee - eb;
    const float alpha32 = (float)a.alpha;
    res_setup<N>(m, sm, st, eb, ne, mx.pot32, alpha32);
    double* sm64 = (double*)(sm + 8 * st);  // FP64 staging of the refinement
    const Fac<double> fac64 = fac_of<double>(m);
    const double* pot64 = (const double*)a.pot;
    const double* bp[2] = {(const double*)a.b[0], (const double*)a.b[1]};
    double* xp[2] = {(double*)a.x[0], (double*)a.x[1]};
    const long long nb = (long long)eb * NN, nend = (long long)ee * NN;
    const int kmax = a.kmax;
    int slot = 0;
    unsigned epoch = 0;
    bool ok = true;
    int sweep = 0, inner_total = 0;
    bool conv = false;
    for (;;) {
        // ---- FP64 residual r = unmask(b) - DSS(A_local(unmask(x)))
        const bool applied = (sweep > 0) || !a.x_is_zero;
        if (applied) {
            __syncthreads();  // the staging area overlays the inner solve's planes
            load_dmat_raw<N, double>(sm64, m);
            __syncthreads();
            for (int e0 = eb; e0 < ee; e0 += kmax)
                apply_range<N, double, OP_RES>(
                    sm64, kmax, fac64, pot64, a.alpha, e0, min(kmax, ee - e0),
                    [&](int e, int i, int j, long long flat, double* u) {
                        const long long src = ni_gather_src(m, node_info<N>(m, e, i, j), e, flat);
                        u[0] = xp[0][src];
                        u[1] = xp[1][src];
                    },
                    [&](int, int, int, long long flat, const double* o) {
                        mx.Y64[0][flat] = o[0];
                        mx.Y64[1][flat] = o[1];
                    });
            if (!grid_barrier(a.sync, a.timeout_ns)) return;
        }
        double part = 0.0, partb = 0.0;
        const bool want_b = (sweep == 0) && a.rel_to_b;
#pragma unroll 4
        for (long long idx = nb + threadIdx.x; idx < nend; idx += blockDim.x) {
            const int e = (int)(idx / NN);
            const int node = (int)(idx - (long long)e * NN);
            const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
            const long long src = ni_gather_src(m, ni, e, idx);
            const bool own = ni_owner(ni);
#pragma unroll
            for (int c = 0; c < 2; ++c) {
                const double bv = bp[c][src];
                double r = bv;
                if (applied) r = r - dss_value<N, double, DSS_CONT>(m, mx.Y64[c], ni, e, idx);
                mx.r64[c][idx] = r;
                if (own) {
                    part = fma(r, r, part);
                    if (want_b) partb = fma(bv, bv, partb);
                }
            }
        }
        double rr = 0.0, bbv = 0.0;
        grid_sum2_t<double>(part, partb, w.partials, slot, a.sync, a.timeout_ns, red, ok, rr, bbv);
        slot ^= 1;
        if (!ok) return;
        if (threadIdx.x == 0) {
            const double rn = sqrt(rr);
            if (sweep == 0) sweep_state[0] = want_b ? sqrt(bbv) : rn;
            sweep_state[1] = rn;
            const double r0 = sweep_state[0];
            const bool c = rn < mx.outer_scale * (a.tol * r0 + a.tol) || rn == 0.0;
            sweep_state[2] = (c || sweep >= mx.max_sweeps || inner_total >= a.maxit || !(rn == rn))
                                 ? (c ? 2.0 : 1.0)
                                 : 0.0;
        }
        __syncthreads();
        if (sweep_state[2] != 0.0) {
            conv = sweep_state[2] == 2.0;
            break;
        }
        // ---- FP32 inner solve A d = r on chip; x += d
        const int budget = min(mx.inner_maxit, a.maxit - inner_total);
        double itol = mx.inner_tol;
        if (mx.adaptive) {
            const double need = mx.outer_scale * (a.tol * sweep_state[0] + a.tol) / sweep_state[1];
            itol = fmax(itol, fmin(0.3 * need, 0.5));
        }
        const double* r64c[2] = {mx.r64[0], mx.r64[1]};
        ResOut ir{};
        if (!res_inner<N>(m, cf, sm, st, eb, ne, r64c, sweep_state[1], alpha32, ra.xa, ra.xb, ra.slots, epoch,
                          a.sync, a.timeout_ns, red, budget, (float)itol, xp, ir))
            return;
        inner_total += ir.it;
        ++sweep;
        if (!grid_barrier(a.sync, a.timeout_ns)) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->success = conv ? 1 : 0;
        a.out->n_iter = inner_total;
        a.out->residual = sweep_state[1];
        a.out->status = 0;
        a.out->inner_iters = inner_total;
        a.out->sweeps = sweep;
    }
}

// ---------------------------------------------------------------- launcher
// Plan: one block per SM (fewer for small meshes); fits when a block's
// elements need at most RES_TPB * RES_NPT nodes and RES_PLANES planes of
// shared memory within smem_budget.  kmax64: elements per pass of the FP64
// refinement's staged apply, which overlays planes 8-17 (extended when one
// pass needs more).
template <int N>
bool resident_plan(int E, int sms, size_t smem_budget, int* grid_out, int* st_out, int* kmax64_out,
                   size_t* smem_out)
{
    constexpr int NN = N * N;
    int grid = E < sms ? E : sms;
    if (grid < 1 || grid > 32 * RES_MAXQ) return false;
    const int kres = (E + grid - 1) / grid;
    const int st = kres * NN;
    if (st > RES_TPB * RES_NPT) return false;
    // planes 8-17 double as the FP64 staging area; small blocks need more
    const size_t fixed = (size_t)8 * st * sizeof(float);
    const size_t planes = (size_t)(RES_PLANES - 8) * st * sizeof(float);
    int k64 = kres;
    auto need = [&](int k) {
        const size_t f64 = range_smem_bytes<N, double, OP_RES>(k);
        return fixed + (f64 > planes ? f64 : planes);
    };
    while (k64 > 1 && need(k64) > smem_budget) --k64;
    const size_t smem = need(k64);
    if (smem > smem_budget) return false;
    *grid_out = grid;
    *st_out = st;
    *kmax64_out = k64;
    *smem_out = smem;
    return true;
}

template <int N>
cudaError_t launch_resident(const DevMesh& m, const SolveArgs& a, const KrylovWork<float>& w, const MixedArgs& mx,
                            const float* D32h, const float* S32h, int st, unsigned long long* slots,
                            unsigned long long* xa, unsigned long long* xb, int grid, size_t smem,
                            cudaStream_t stream)
{
    const void* fn = (const void*)k_minres_resident<N>;
    // a per-device function attribute: set on every launch (cheap), so a
    // context on any device of the process gets the opt-in
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    DevMesh mm = m;
    SolveArgs aa = a;
    KrylovWork<float> ww = w;
    MixedArgs xx = mx;
    ResCoef<N> cf;
    for (int q = 0; q < N * N; ++q) {
        cf.D[q] = D32h[q];
        cf.S[q] = S32h[q];
    }
    ResArgs ra{st, xa, xb, slots};
    void* args[] = {&mm, &aa, &ww, &xx, &cf, &ra};
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(RES_TPB), args, smem, stream);
}

#define SEM_INSTANTIATE_RESIDENT(NV)                                                                           \
    template bool resident_plan<NV>(int, int, size_t, int*, int*, int*, size_t*);                             \
    template cudaError_t launch_resident<NV>(const DevMesh&, const SolveArgs&, const KrylovWork<float>&,      \
                                             const MixedArgs&, const float*, const float*, int,               \
                                             unsigned long long*, unsigned long long*, unsigned long long*, int,   \
                                             size_t, cudaStream_t);

}  // namespace semgb
