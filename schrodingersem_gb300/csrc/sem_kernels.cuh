// Standalone kernels (operator apply, assembly, masking, dots, stage
// combinations) and their launchers.  Included by the sem_inst_*.cu units,
// which instantiate them for a list of polynomial degrees.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "sem_apply_bulk.cuh"
#include "sem_device.cuh"
#include "sem_solvers.cuh"

namespace semgb {

// element-local operator, input gathered with unmask semantics when GATHER
template <int N, typename T, int OP, bool GATHER>
__global__ void __launch_bounds__(geo_tpb(N))
    k_apply(DevMesh m, const T* __restrict__ pot, T alpha, const T* __restrict__ in0,
            const T* __restrict__ in1, T* __restrict__ y0, T* __restrict__ y1)
{
    __shared__ ApplySmem<N, T, OP> s;
    load_dmat(s, m);
    __syncthreads();
    const Fac<T> fac = fac_of<T>(m);
    const int e0 = blockIdx.x * geo_k(N);
    apply_chunk<N, T, OP>(
        s, fac, pot, alpha, e0, m.E,
        [&](int e, int i, int j, long long flat, T* u) {
            long long src = flat;
            if (GATHER) src = ni_gather_src(m, node_info<N>(m, e, i, j), e, flat);
            u[0] = in0[src];
            if (op_nc<OP>() == 2) u[op_nc<OP>() - 1] = in1[src];
        },
        [&](int e, int i, int j, long long flat, const T* o) {
            y0[flat] = o[0];
            if (op_nc<OP>() == 2) y1[flat] = o[op_nc<OP>() - 1];
        });
}

template <int N, typename T, int MODE>
__global__ void k_dss(DevMesh m, const T* __restrict__ Y, T* __restrict__ out, T scale)
{
    constexpr int NN = N * N;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < m.n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
        out[idx] = scale * dss_value<N, T, MODE>(m, Y, ni, e, idx);
    }
}

// In-place assembly of element-local values (the apply's own output) that
// touches only the element rings, from precomputed tables: every
// interior-side node pair (owner, other), every boundary-side copy, then
// every corner node over its copies.  One item owns all copies of its
// global node, so no two threads write the same copy.  Sums run in the order
// dss_value uses (owner + other on sides; 0 + copies in connected_elements
// order at corners), so the result equals k_dss<MODE> with scale 1 bit for
// bit.  Element interiors are final as the apply wrote them.
template <int N, typename T, int MODE>
__global__ void k_ring(DevMesh m, long long np, T* __restrict__ a0, T* __restrict__ a1)
{
    const long long nb = m.n_bnd;
    const long long total = np + nb + m.n_nodes;
    T* planes[2] = {a0, a1};
    const long long stride = (long long)gridDim.x * blockDim.x;
    // side pairs, four per thread with their loads issued together
    for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < np; i0 += 4 * stride) {
        int2 pr[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const long long i = i0 + q * stride;
            pr[q] = i < np ? __ldg(m.edge_pairs + i) : make_int2(-1, -1);
        }
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            T* a = planes[c];
            if (!a) continue;
            T x[4], y[4];
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (pr[q].x >= 0) {
                    x[q] = a[pr[q].x];
                    y[q] = a[pr[q].y];
                }
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (pr[q].x >= 0) {
                    const T v = x[q] + y[q];
                    a[pr[q].x] = v;
                    a[pr[q].y] = MODE == DSS_MASK ? T(0) : v;
                }
        }
    }
    for (long long it = np + blockIdx.x * (long long)blockDim.x + threadIdx.x; it < total; it += stride) {
        if (it < np + nb) {
            if (MODE == DSS_SUM) continue;
            const int f = __ldg(m.bnd_flat + (it - np));
#pragma unroll
            for (int q = 0; q < 2; ++q)
                if (planes[q]) planes[q][f] = T(0);
        } else {
            // corner node: its copies in CSR order from one padded row (two
            // dependent loads: the row, the values), else the CSR
            const int node = (int)(it - np - nb);
            const int4* row = reinterpret_cast<const int4*>(m.node_nb + (size_t)node * CORNER_NB_MAX);
            int f[CORNER_NB_MAX];
#pragma unroll
            for (int h = 0; h < CORNER_NB_MAX / 4; ++h) {
                const int4 v = __ldg(row + h);
                f[4 * h] = v.x;
                f[4 * h + 1] = v.y;
                f[4 * h + 2] = v.z;
                f[4 * h + 3] = v.w;
            }
            const bool bnd = __ldg(m.node_bnd + node) != 0;
            if (f[0] == -2) {
                const int q0 = __ldg(m.node_ptr + node), q1 = __ldg(m.node_ptr + node + 1);
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    T* a = planes[q];
                    if (!a) continue;
                    if (bnd) {
                        if (MODE != DSS_SUM)
                            for (int t = q0; t < q1; ++t) a[__ldg(m.node_flat + t)] = T(0);
                        continue;
                    }
                    T sum = T(0);
                    for (int t = q0; t < q1; ++t) sum += a[__ldg(m.node_flat + t)];
                    for (int t = q0; t < q1; ++t)
                        a[__ldg(m.node_flat + t)] = (MODE == DSS_MASK && t != q0) ? T(0) : sum;
                }
                continue;
            }
            if (f[0] < 0) continue;  // no copies
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                T* a = planes[q];
                if (!a) continue;
                if (bnd) {
                    if (MODE != DSS_SUM)
#pragma unroll
                        for (int k = 0; k < CORNER_NB_MAX; ++k)
                            if (f[k] >= 0) a[f[k]] = T(0);
                    continue;
                }
                T v[CORNER_NB_MAX];
#pragma unroll
                for (int k = 0; k < CORNER_NB_MAX; ++k) v[k] = f[k] >= 0 ? a[f[k]] : T(0);
                T sum = T(0);
#pragma unroll
                for (int k = 0; k < CORNER_NB_MAX; ++k)
                    if (f[k] >= 0) sum += v[k];
#pragma unroll
                for (int k = 0; k < CORNER_NB_MAX; ++k)
                    if (f[k] >= 0) a[f[k]] = (MODE == DSS_MASK && k != 0) ? T(0) : sum;
            }
        }
    }
}

// unmask in place: non-owner copies read owner copies, which are never written
template <int N, typename T>
__global__ void k_unmask(DevMesh m, T* a)
{
    constexpr int NN = N * N;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < m.n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
        const long long src = ni_gather_src(m, ni, e, idx);
        if (src != idx) a[idx] = a[src];
    }
}

template <int N, typename T>
__global__ void k_mask(DevMesh m, T* a)
{
    constexpr int NN = N * N;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < m.n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
        if (ni.kind != 0 && (ni_boundary(ni) || !ni_owner(ni))) a[idx] = T(0);
    }
}

// owner-weighted dot: block partials
template <int N>
__global__ void k_dot(DevMesh m, const double* __restrict__ a, const double* __restrict__ b,
                      double* part)
{
    __shared__ double red[34];
    constexpr int NN = N * N;
    double s = 0.0;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < m.n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
        if (ni_owner(ni)) s = fma(a[idx], b[idx], s);
    }
    s = block_sum(s, red);
    if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// v = gather(p + c0 z0 + c1 z1 + ...) then the f closure -> element-local y
template <int N>
__global__ void __launch_bounds__(geo_tpb(N))
    k_combo_f(DevMesh m, const double* __restrict__ V, const double* __restrict__ p, ZList zl,
              double* y)
{
    __shared__ ApplySmem<N, double, OP_F> s;
    load_dmat(s, m);
    __syncthreads();
    const int nz = zl.nz;
    const long long n = m.n;
    const Fac<double> fac = fac_of<double>(m);
    apply_chunk<N, double, OP_F>(
        s, fac, V, 0.0, blockIdx.x * geo_k(N), m.E,
        [&](int e, int i, int j, long long flat, double* u) {
            const long long src = ni_gather_src(m, node_info<N>(m, e, i, j), e, flat);
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                double v = p[q * n + src];
                for (int l = 0; l < nz; ++l) v = v + zl.c[l] * zl.z[l][q * n + src];
                u[q] = v;
            }
        },
        [&](int e, int i, int j, long long flat, const double* o) {
            y[flat] = o[0];
            y[n + flat] = o[1];
        });
}

// p_out = unmask(p_in + (c0 z0 + c1 z1 + ...)), both planes
template <int N>
__global__ void k_update(DevMesh m, const double* __restrict__ p_in, ZList zl,
                         double* __restrict__ p_out)
{
    constexpr int NN = N * N;
    const int nz = zl.nz;
    const long long n = m.n;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const long long src = ni_gather_src(m, node_info<N>(m, e, node % N, node / N), e, idx);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            double acc = zl.c[0] * zl.z[0][q * n + src];
            for (int l = 1; l < nz; ++l) acc = acc + zl.c[l] * zl.z[l][q * n + src];
            p_out[q * n + idx] = p_in[q * n + src] + acc;
        }
    }
}

// ------------------------------------------------- learned stage guess
// r = unmask(b) - DSS_cont(Y) for two planes: the residual of a guess whose
// element-local operator output is Y, in the continuous format
template <int N>
__global__ void k_resid_cont(DevMesh m, const double* __restrict__ b, const double* __restrict__ Y,
                             double* __restrict__ r)
{
    constexpr int NN = N * N;
    const long long n = m.n;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
        const long long src = ni_gather_src(m, ni, e, idx);
#pragma unroll
        for (int q = 0; q < 2; ++q) r[q * n + idx] = b[q * n + src] - dss_value<N, double, DSS_CONT>(m, Y + q * n, ni, e, idx);
    }
}

// One warp per element.  rho_e = RMS of the residual over the element's
// nodes (both planes), at least rho_floor (elements the residual has not
// reached get small features and targets instead of scaled round-off),
// mbar_e = mean lumped mass w_i w_j J of the element;
// features (BF16, row e):
//   [r_re / rho, r_im / rho, alpha V, (w_i w_j J) / alpha]   (4 N^2 values)
// and the element's solution scale sigma_e = rho_e / mbar_e (the size of
// M^-1 r, the error a mass-dominated residual of size rho points to)
template <int N>
__global__ void k_features(DevMesh m, const double* __restrict__ r, const double* __restrict__ V, double alpha,
                           double rho_floor, __nv_bfloat16* __restrict__ x, float* __restrict__ sigma)
{
    constexpr int NN = N * N;
    const long long n = m.n;
    const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (e >= m.E) return;
    const long long base = (long long)e * NN;
    double s = 0.0, ms = 0.0;
    for (int k = lane; k < NN; k += 32) {
        const double a = r[base + k], b = r[n + base + k];
        s += a * a + b * b;
        ms += m.mass[base + k];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        ms += __shfl_xor_sync(0xffffffffu, ms, o);
    }
    const double rho = fmax(sqrt(s / (2.0 * NN)), rho_floor);
    const double inv = 1.0 / rho;
    const double inv_alpha = 1.0 / alpha;  // one FP64 division per thread, not per node
    __nv_bfloat16* row = x + (long long)e * 4 * NN;
    for (int k = lane; k < NN; k += 32) {
        row[k] = __float2bfloat16((float)(r[base + k] * inv));
        row[NN + k] = __float2bfloat16((float)(r[n + base + k] * inv));
        row[2 * NN + k] = __float2bfloat16((float)(alpha * V[base + k]));
        row[3 * NN + k] = __float2bfloat16((float)(m.mass[base + k] * inv_alpha));
    }
    if (lane == 0) sigma[e] = (float)(rho * NN / ms);
}

// training target of element e: (z - z_guess) / sigma_e at every node, with
// the solution read at the owner copies (continuous values)
template <int N>
__global__ void k_targets(DevMesh m, const double* __restrict__ z, const double* __restrict__ zg,
                          const float* __restrict__ sigma, float* __restrict__ t)
{
    constexpr int NN = N * N;
    const long long n = m.n;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
        const long long src = ni_gather_src(m, ni, e, idx);
        const double inv = 1.0 / (double)sigma[e];
        float* row = t + (long long)e * 2 * NN;
        row[node] = (float)((z[src] - zg[src]) * inv);
        row[NN + node] = (float)((z[n + src] - zg[n + src]) * inv);
    }
}

// z_out = z_guess + sigma_e * delta_e in the masked format: the owner copy
// of each node takes its element's correction, other copies and the
// boundary stay zero (z_guess is masked)
template <int N>
__global__ void k_correct(DevMesh m, const double* __restrict__ zg, const float* __restrict__ sigma,
                          const float* __restrict__ delta, double* __restrict__ zo)
{
    constexpr int NN = N * N;
    const long long n = m.n;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
        if (!ni_owner(ni) || ni_boundary(ni)) {
            zo[idx] = 0.0;
            zo[n + idx] = 0.0;
            continue;
        }
        const double s = (double)sigma[e];
        const float* row = delta + (long long)e * 2 * NN;
        zo[idx] = zg[idx] + s * (double)row[node];
        zo[n + idx] = zg[n + idx] + s * (double)row[NN + node];
    }
}

// ------------------------------------------------------------- launchers

inline int grid_for(long long work, int tpb, int cap = 152 * 32)
{
    long long g = (work + tpb - 1) / tpb;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

template <int N>
cudaError_t launch_apply(const DevMesh& m, int op, bool fp32, const void* pot, double alpha,
                         const void* in0, const void* in1, void* y0, void* y1, bool gather,
                         cudaStream_t st)
{
    const int grid = (m.E + geo_k(N) - 1) / geo_k(N);
    const int tpb = geo_tpb(N);
#define SEM_APPLY_CASE(T, OPK)                                                                    \
    if (gather)                                                                                   \
        k_apply<N, T, OPK, true><<<grid, tpb, 0, st>>>(m, (const T*)pot, (T)alpha, (const T*)in0, \
                                                       (const T*)in1, (T*)y0, (T*)y1);            \
    else                                                                                          \
        k_apply<N, T, OPK, false><<<grid, tpb, 0, st>>>(m, (const T*)pot, (T)alpha,               \
                                                        (const T*)in0, (const T*)in1, (T*)y0,     \
                                                        (T*)y1);
    if (!fp32) {
        switch (op) {
            case OP_LAPLACE: SEM_APPLY_CASE(double, OP_LAPLACE) break;
            case OP_HELM: SEM_APPLY_CASE(double, OP_HELM) break;
            case OP_MASS: SEM_APPLY_CASE(double, OP_MASS) break;
            case OP_RES: SEM_APPLY_CASE(double, OP_RES) break;
            case OP_F: SEM_APPLY_CASE(double, OP_F) break;
            default: return cudaErrorInvalidValue;
        }
    } else {
        switch (op) {
            case OP_RES: SEM_APPLY_CASE(float, OP_RES) break;
            case OP_LAPLACE: SEM_APPLY_CASE(float, OP_LAPLACE) break;
            default: return cudaErrorInvalidValue;
        }
    }
#undef SEM_APPLY_CASE
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_apply_bulk(const DevMesh& m, int op, bool fp32, const void* pot, double alpha, const void* in0,
                              const void* in1, void* y0, void* y1, bool gather, bool pair_asm, bool geo,
                              long long timeout_ns, cudaStream_t st)
{
#define SEM_BULK_CASE(T, OPK)                                                                                 \
    return gather ? launch_apply_bulk_t<N, T, OPK, true>(m, (const T*)pot, (T)alpha, (const T*)in0,           \
                                                         (const T*)in1, (T*)y0, (T*)y1, pair_asm, geo,        \
                                                         timeout_ns, st)                                      \
                  : launch_apply_bulk_t<N, T, OPK, false>(m, (const T*)pot, (T)alpha, (const T*)in0,          \
                                                          (const T*)in1, (T*)y0, (T*)y1, pair_asm, geo,       \
                                                          timeout_ns, st);
    if (!fp32) return cudaErrorInvalidValue;  // FP64 applies are FP64-pipe bound: one-pass kernel
    switch (op) {
        case OP_RES: SEM_BULK_CASE(float, OP_RES)
        default: return cudaErrorInvalidValue;
    }
#undef SEM_BULK_CASE
}

template <int N>
cudaError_t launch_dss(const DevMesh& m, bool fp32, int mode, double scale, const void* y,
                       void* out, cudaStream_t st)
{
    const int tpb = 256;
    const int grid = grid_for(m.n, tpb);
#define SEM_DSS_CASE(T)                                                                                     \
    switch (mode) {                                                                                         \
        case DSS_SUM: k_dss<N, T, DSS_SUM><<<grid, tpb, 0, st>>>(m, (const T*)y, (T*)out, (T)scale); break;   \
        case DSS_MASK: k_dss<N, T, DSS_MASK><<<grid, tpb, 0, st>>>(m, (const T*)y, (T*)out, (T)scale); break; \
        default: k_dss<N, T, DSS_CONT><<<grid, tpb, 0, st>>>(m, (const T*)y, (T*)out, (T)scale); break;       \
    }
    if (fp32) {
        SEM_DSS_CASE(float)
    } else {
        SEM_DSS_CASE(double)
    }
#undef SEM_DSS_CASE
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_unmask(const DevMesh& m, bool fp32, void* a, cudaStream_t st)
{
    const int grid = grid_for(m.n, 256);
    if (fp32) k_unmask<N, float><<<grid, 256, 0, st>>>(m, (float*)a);
    else k_unmask<N, double><<<grid, 256, 0, st>>>(m, (double*)a);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_mask(const DevMesh& m, bool fp32, void* a, cudaStream_t st)
{
    const int grid = grid_for(m.n, 256);
    if (fp32) k_mask<N, float><<<grid, 256, 0, st>>>(m, (float*)a);
    else k_mask<N, double><<<grid, 256, 0, st>>>(m, (double*)a);
    return cudaGetLastError();
}

// three owner-weighted dots of two-plane vectors at once: part[3 blk + q] =
// (a.a, a.b, b.b) over both planes (fixed order), FP64 sums; b FP64 or FP32
template <int N, typename TB>
__global__ void k_dot3(DevMesh m, const double* __restrict__ a, const TB* __restrict__ b, double* part)
{
    __shared__ double red[34];
    constexpr int NN = N * N;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < m.n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
        if (ni_owner(ni)) {
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const double x = a[q * m.n + idx], y = (double)b[q * m.n + idx];
                s0 = fma(x, x, s0);
                s1 = fma(x, y, s1);
                s2 = fma(y, y, s2);
            }
        }
    }
    s0 = block_sum(s0, red);
    s1 = block_sum(s1, red);
    s2 = block_sum(s2, red);
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = s0;
        part[3 * blockIdx.x + 1] = s1;
        part[3 * blockIdx.x + 2] = s2;
    }
}

template <int N>
cudaError_t launch_dot3(const DevMesh& m, const double* a, const double* b, double* part, int max_blocks,
                        int* blocks_used, cudaStream_t st)
{
    const int grid = grid_for(m.n, 256, max_blocks);
    *blocks_used = grid;
    k_dot3<N, double><<<grid, 256, 0, st>>>(m, a, b, part);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_dot3_f32(const DevMesh& m, const double* a, const float* b, double* part, int max_blocks,
                            int* blocks_used, cudaStream_t st)
{
    const int grid = grid_for(m.n, 256, max_blocks);
    *blocks_used = grid;
    k_dot3<N, float><<<grid, 256, 0, st>>>(m, a, b, part);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_dot(const DevMesh& m, const double* a, const double* b, double* part,
                       int max_blocks, int* blocks_used, cudaStream_t st)
{
    const int grid = grid_for(m.n, 256, max_blocks);
    *blocks_used = grid;
    k_dot<N><<<grid, 256, 0, st>>>(m, a, b, part);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_combo_f(const DevMesh& m, const double* V, const double* p, const ZList& zl,
                           double* y, cudaStream_t st)
{
    const int grid = (m.E + geo_k(N) - 1) / geo_k(N);
    k_combo_f<N><<<grid, geo_tpb(N), 0, st>>>(m, V, p, zl, y);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_update(const DevMesh& m, const double* p_in, const ZList& zl, double* p_out,
                          cudaStream_t st)
{
    const int grid = grid_for(m.n, 256);
    k_update<N><<<grid, 256, 0, st>>>(m, p_in, zl, p_out);
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_ring(const DevMesh& m, bool fp32, int mode, void* a0, void* a1, bool cross_only,
                        cudaStream_t st)
{
    const int tpb = 256;
    const long long np = cross_only ? m.n_pairs_x : m.n_pairs;
    const int grid = grid_for(np + m.n_bnd + m.n_nodes, tpb);
#define SEM_RING_CASE(T)                                                                                  \
    switch (mode) {                                                                                       \
        case DSS_SUM: k_ring<N, T, DSS_SUM><<<grid, tpb, 0, st>>>(m, np, (T*)a0, (T*)a1); break;         \
        case DSS_MASK: k_ring<N, T, DSS_MASK><<<grid, tpb, 0, st>>>(m, np, (T*)a0, (T*)a1); break;       \
        default: k_ring<N, T, DSS_CONT><<<grid, tpb, 0, st>>>(m, np, (T*)a0, (T*)a1); break;             \
    }
    if (fp32) {
        SEM_RING_CASE(float)
    } else {
        SEM_RING_CASE(double)
    }
#undef SEM_RING_CASE
    return cudaGetLastError();
}

template <int N>
cudaError_t launch_learn(const DevMesh& m, const LearnArgs& a, cudaStream_t st)
{
    const int grid = grid_for(m.n, 256);
    switch (a.what) {
        case LEARN_RESID: k_resid_cont<N><<<grid, 256, 0, st>>>(m, a.b, a.Y, a.r); break;
        case LEARN_FEATURES:
            k_features<N><<<(m.E + 7) / 8, 256, 0, st>>>(m, a.r, a.V, a.alpha, a.rho_floor, (__nv_bfloat16*)a.x,
                                                           a.sigma);
            break;
        case LEARN_TARGETS: k_targets<N><<<grid, 256, 0, st>>>(m, a.z, a.zg, a.sigma, a.t); break;
        case LEARN_CORRECT: k_correct<N><<<grid, 256, 0, st>>>(m, a.zg, a.sigma, a.delta, a.zo); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace semgb

#define SEM_INSTANTIATE(NV)                                                                          \
    namespace semgb {                                                                                \
    template cudaError_t launch_apply<NV>(const DevMesh&, int, bool, const void*, double,            \
                                          const void*, const void*, void*, void*, bool,              \
                                          cudaStream_t);                                             \
    template cudaError_t launch_dss<NV>(const DevMesh&, bool, int, double, const void*, void*,       \
                                        cudaStream_t);                                               \
    template cudaError_t launch_ring<NV>(const DevMesh&, bool, int, void*, void*, bool, cudaStream_t); \
    template cudaError_t launch_apply_bulk<NV>(const DevMesh&, int, bool, const void*, double,       \
                                               const void*, const void*, void*, void*, bool, bool,   \
                                               bool, long long, cudaStream_t);                       \
    template cudaError_t launch_unmask<NV>(const DevMesh&, bool, void*, cudaStream_t);               \
    template cudaError_t launch_mask<NV>(const DevMesh&, bool, void*, cudaStream_t);                 \
    template cudaError_t launch_dot<NV>(const DevMesh&, const double*, const double*, double*, int,  \
                                        int*, cudaStream_t);                                         \
    template cudaError_t launch_dot3<NV>(const DevMesh&, const double*, const double*, double*, int, \
                                         int*, cudaStream_t);                                        \
    template cudaError_t launch_dot3_f32<NV>(const DevMesh&, const double*, const float*, double*,   \
                                             int, int*, cudaStream_t);                               \
    template cudaError_t launch_combo_f<NV>(const DevMesh&, const double*, const double*,            \
                                            const ZList&, double*, cudaStream_t);                    \
    template cudaError_t launch_update<NV>(const DevMesh&, const double*, const ZList&, double*,     \
                                           cudaStream_t);                                            \
    template int solver_plan<NV>(int, bool, int, int, size_t, int*, size_t*);                        \
    template cudaError_t launch_learn<NV>(const DevMesh&, const LearnArgs&, cudaStream_t);           \
    template cudaError_t launch_solver<NV>(const DevMesh&, const SolveArgs&, const void*,            \
                                           const MixedArgs*, int, size_t, cudaStream_t);             \
    }
