// Device-side building blocks for the sm_103a spectral-element kernels.
//
// Data layout: a field is E element blocks of N*N values, column-major
// inside the block: node (i,j) of element e at flat index e*N*N + j*N + i
// (the reference's std::vector<arma::Mat> laid end to end).
#pragma once
#include <cfloat>
#include <cstdint>

#include "sem_internal.h"

namespace semgb {

// ---------------------------------------------------------------- geometry
// Elements per block-chunk (K) and threads per block (TPB) for each N: one
// thread per element-local node, K elements side by side, TPB a multiple of
// 32 chosen to waste as few lanes as possible.
__host__ __device__ constexpr int geo_k(int N)
{
    return N <= 9 ? 256 / (N * N) : N == 10 ? 5 : N == 11 ? 4 : N <= 13 ? 3 : N <= 16 ? 2 : 1;
}
__host__ __device__ constexpr int geo_tpb(int N)
{
    return ((geo_k(N) * N * N + 31) / 32) * 32;
}

// blocks per SM the persistent kernels are compiled for (caps registers at 128)
__host__ __device__ constexpr int geo_minb(int N)
{
    return geo_tpb(N) <= 256 ? 2 : 1;
}

template <int OP>
__host__ __device__ constexpr int op_nc()
{
    return (OP == OP_RES || OP == OP_F) ? 2 : 1;
}

template <typename T>
struct Fac {
    const T *g11, *g12, *g22, *mass;
};

template <typename T>
__host__ __device__ inline Fac<T> fac_of(const DevMesh& m);
template <>
__host__ __device__ inline Fac<double> fac_of<double>(const DevMesh& m)
{
    return Fac<double>{m.g11, m.g12, m.g22, m.mass};
}
template <>
__host__ __device__ inline Fac<float> fac_of<float>(const DevMesh& m)
{
    return Fac<float>{m.g11f, m.g12f, m.g22f, m.massf};
}
template <typename T>
__device__ inline const T* dmat_of(const DevMesh& m);
template <>
__device__ inline const double* dmat_of<double>(const DevMesh& m) { return m.D64; }
template <>
__device__ inline const float* dmat_of<float>(const DevMesh& m) { return m.D32; }

// ------------------------------------------------------- node classification
// kind 0: element interior; 1: side sc, position k; 2: corner sc.
struct NodeInfo {
    int kind, sc, k, flags;
};

template <int N>
__device__ __forceinline__ NodeInfo node_info(const DevMesh& m, int e, int i, int j)
{
    NodeInfo r;
    const bool ib = (i == 0) | (i == N - 1);
    const bool jb = (j == 0) | (j == N - 1);
    r.k = 0;
    if (ib && jb) {
        r.kind = 2;
        r.sc = (j == 0) ? (i == 0 ? 0 : 1) : (i == 0 ? 3 : 2);
    } else if (jb) {
        r.kind = 1;
        r.sc = (j == 0) ? 0 : 2;
        r.k = i;
    } else if (ib) {
        r.kind = 1;
        r.sc = (i == N - 1) ? 1 : 3;
        r.k = j;
    } else {
        r.kind = 0;
        r.sc = 0;
    }
    r.flags = (r.kind == 0) ? 0 : __ldg(m.flags + e);
    return r;
}

// is this copy the one the reference's dot() counts (dot.hpp:11-61)?
__device__ __forceinline__ bool ni_owner(const NodeInfo& ni)
{
    if (ni.kind == 0) return true;
    if (ni.kind == 1) return (ni.flags >> ni.sc) & 1;
    return (ni.flags >> (8 + ni.sc)) & 1;
}

__device__ __forceinline__ bool ni_boundary(const NodeInfo& ni)
{
    if (ni.kind == 0) return false;
    if (ni.kind == 1) return (ni.flags >> (4 + ni.sc)) & 1;
    return (ni.flags >> (12 + ni.sc)) & 1;
}

// a side copy with no partner (a side on a Neumann boundary)
__device__ __forceinline__ bool ni_lone(const NodeInfo& ni)
{
    return ni.kind == 1 && ((ni.flags >> (16 + ni.sc)) & 1);
}

// flat index whose value unmask() copies into this node: the owner copy for
// non-owner copies of interior sides/corners (unmask.hpp:12-36), else itself.
__device__ __forceinline__ long long ni_gather_src(const DevMesh& m, const NodeInfo& ni, int e,
                                                   long long flat)
{
    if (ni.kind == 0 || ni_owner(ni) || ni_boundary(ni)) return flat;
    if (ni.kind == 1)
        return (long long)__ldg(m.side_base + 4 * e + ni.sc) +
               (long long)ni.k * __ldg(m.side_step + 4 * e + ni.sc);
    return __ldg(m.corner_src + 4 * e + ni.sc);
}

template <typename T>
__device__ __forceinline__ T ldcg(const T* p) { return __ldcg(p); }

// assembled value at a node (global_sum.hpp:13-63 + mask.hpp:16-28 by mode).
// Values of other elements are read with ld.cg: inside the persistent
// kernels they were written by other blocks in the previous phase.
// The index tables of a node are read before its flags are tested, so a side
// copy costs two dependent loads (tables, other copy) and a corner copy two
// (its copy list, the copies).
template <int N, typename T, int MODE>
__device__ __forceinline__ T dss_value(const DevMesh& m, const T* Y, const NodeInfo& ni, int e,
                                       long long flat)
{
    const T own = ldcg(Y + flat);
    if (ni.kind == 0) return own;
    if (ni.kind == 1) {
        const int sb = __ldg(m.side_base + 4 * e + ni.sc), ss = __ldg(m.side_step + 4 * e + ni.sc);
        if (ni_boundary(ni)) return MODE == DSS_SUM ? own : T(0);
        if (MODE == DSS_MASK && !ni_owner(ni)) return T(0);
        if (ni_lone(ni)) return own;
        return own + ldcg(Y + ((long long)sb + (long long)ni.k * ss));  // owner + other in either copy: same bits
    }
    const int* cl = m.corner_nb + (size_t)(4 * e + ni.sc) * CORNER_NB_MAX;
    int q[CORNER_NB_MAX];
#pragma unroll
    for (int k = 0; k < CORNER_NB_MAX; ++k) q[k] = __ldg(cl + k);
    if (ni_boundary(ni)) return MODE == DSS_SUM ? own : T(0);
    if (MODE == DSS_MASK && !ni_owner(ni)) return T(0);
    T s = T(0);  // csum = 0, then += in connected_elements order (global_sum.hpp:56-59)
    if (q[0] == -2) {  // more copies than the table holds
        const int node = __ldg(m.corner_node + 4 * e + ni.sc);
        const int q0 = __ldg(m.node_ptr + node), q1 = __ldg(m.node_ptr + node + 1);
        for (int k = q0; k < q1; ++k) s += ldcg(Y + __ldg(m.node_flat + k));
        return s;
    }
    T v[CORNER_NB_MAX];
#pragma unroll
    for (int k = 0; k < CORNER_NB_MAX; ++k) v[k] = q[k] >= 0 ? ldcg(Y + q[k]) : T(0);
#pragma unroll
    for (int k = 0; k < CORNER_NB_MAX; ++k)
        if (q[k] >= 0) s += v[k];
    return s;
}

// ------------------------------------------------------------ element apply
template <int N, typename T, int OP>
struct ApplySmem {
    static constexpr int NN = N * N;
    static constexpr int K = geo_k(N);
    static constexpr int NC = op_nc<OP>();
    T D[NN];
    T u[NC][K * NN];
    T f1[NC][K * NN];
    T f2[NC][K * NN];
};

template <int N, typename T, int OP>
__device__ __forceinline__ void load_dmat(ApplySmem<N, T, OP>& s, const DevMesh& m)
{
    const T* D = dmat_of<T>(m);
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) s.D[t] = D[t];
}

// One block-wide pass of the fused element operator over elements
// [e0, min(e0+K, e_end)).  Every thread of the block must call it (it holds
// __syncthreads).  load(e,i,j,flat,u[NC]) supplies the node's input values;
// store(e,i,j,flat,out[NC]) receives the element-local result.
//
// Weak Laplacian with premultiplied factors (glaplace.hpp:16-28 rewritten
// with g11 = w_i w_j A, g12 = w_i w_j B, g22 = w_i w_j C):
//   f1 = g11 u_xi - g12 u_eta,   f2 = g22 u_eta - g12 u_xi
//   lap(i,j) = sum_k D(k,i) f1(k,j) + sum_k D(k,j) f2(i,k)
// Mass term (W (u%V) W) % J = (w_i w_j J) V u.
template <int N, typename T, int OP, class Load, class Store>
__device__ __forceinline__ void apply_chunk(ApplySmem<N, T, OP>& s, const Fac<T>& fac,
                                            const T* __restrict__ pot, T alpha, int e0, int e_end,
                                            Load&& load, Store&& store)
{
    constexpr int NN = N * N;
    constexpr int K = geo_k(N);
    constexpr int NC = op_nc<OP>();
    const int t = threadIdx.x;
    const int le = t / NN;
    const int node = t - le * NN;
    const int i = node % N, j = node / N;
    const int e = e0 + le;
    const bool active = (le < K) && (e < e_end);
    const long long flat = (long long)e * NN + node;
    T u[NC];
    T g11 = T(0), g12 = T(0), g22 = T(0), ms = T(0), pv = T(0);
    if (active) {
        if (OP != OP_MASS) {
            g11 = __ldg(fac.g11 + flat);
            g12 = __ldg(fac.g12 + flat);
            g22 = __ldg(fac.g22 + flat);
        }
        if (OP != OP_LAPLACE) ms = __ldg(fac.mass + flat);
        if (OP == OP_HELM || OP == OP_RES || OP == OP_F) pv = __ldg(pot + flat);
        load(e, i, j, flat, u);
    }
    if (OP == OP_MASS) {
        if (active) {
            T o[NC];
            o[0] = ms * u[0];
            store(e, i, j, flat, o);
        }
        return;
    }
    if (active) {
#pragma unroll
        for (int c = 0; c < NC; ++c) s.u[c][le * NN + node] = u[c];
    }
    __syncthreads();
    if (active) {
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T* uc = &s.u[c][le * NN];
            T ur = T(0), us = T(0);
#pragma unroll
            for (int k = 0; k < N; ++k) {
                ur = fma(s.D[i * N + k], uc[k + j * N], ur);  // (D u)(i,j)
                us = fma(s.D[j * N + k], uc[i + k * N], us);  // (u D^T)(i,j)
            }
            s.f1[c][le * NN + node] = g11 * ur - g12 * us;
            s.f2[c][le * NN + node] = g22 * us - g12 * ur;
        }
    }
    __syncthreads();
    if (active) {
        T lap[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T* f1 = &s.f1[c][le * NN];
            const T* f2 = &s.f2[c][le * NN];
            T a = T(0);
#pragma unroll
            for (int k = 0; k < N; ++k) a = fma(s.D[k * N + i], f1[k + j * N], a);
#pragma unroll
            for (int k = 0; k < N; ++k) a = fma(s.D[k * N + j], f2[i + k * N], a);
            lap[c] = a;
        }
        T o[NC];
        if (OP == OP_LAPLACE) {
            o[0] = lap[0];
        } else if (OP == OP_HELM) {
            o[0] = lap[0] + (ms * pv) * u[0];
        } else if (OP == OP_RES) {
            const T mv = ms * pv;
            const T Lv = lap[NC - 1] + mv * u[NC - 1];
            const T Lu = lap[0] + mv * u[0];
            o[0] = ms * u[0] + alpha * Lv;
            o[NC - 1] = alpha * Lu - ms * u[NC - 1];
        } else {  // OP_F
            const T mv = ms * pv;
            o[0] = -(lap[NC - 1] + mv * u[NC - 1]);
            o[NC - 1] = -(lap[0] + mv * u[0]);
        }
        store(e, i, j, flat, o);
    }
    __syncthreads();
}

// ----------------------------------------------- range-staged element apply
// The persistent solvers give every block a contiguous element range and
// stage up to kmax elements of it in dynamic shared memory at once, every
// thread looping over several nodes in each sub-phase.  All loads of the
// staged range are issued before the first barrier, so one pass costs one
// memory latency instead of one per small chunk.
// Shared layout (type T): D[NN] | u[NC][kmax*NN] | f1[NC][kmax*NN] | f2[NC][kmax*NN]
template <int N, typename T, int OP>
__host__ __device__ constexpr size_t range_smem_bytes(int kmax)
{
    return sizeof(T) * ((size_t)N * N + 3ull * op_nc<OP>() * (size_t)kmax * N * N);
}

template <int N, typename T>
__device__ __forceinline__ void load_dmat_raw(T* sm, const DevMesh& m)
{
    const T* D = dmat_of<T>(m);
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) sm[t] = D[t];
}

template <int N, typename T, int OP, bool POST, class Load, class Post, class Store>
__device__ __forceinline__ void apply_range_post(T* sm, int kmax, const Fac<T>& fac,
                                                 const T* __restrict__ pot, T alpha, int e0, int ne,
                                                 Load&& load, Post&& post, Store&& store);

// One block-wide pass over elements [e0, e0+ne), ne <= kmax.  Every thread
// of the block must call it.  Same operator and callbacks as apply_chunk.
template <int N, typename T, int OP, class Load, class Store>
__device__ __forceinline__ void apply_range(T* sm, int kmax, const Fac<T>& fac,
                                            const T* __restrict__ pot, T alpha, int e0, int ne,
                                            Load&& load, Store&& store)
{
    apply_range_post<N, T, OP, false>(
        sm, kmax, fac, pot, alpha, e0, ne,
        [&](int e, int i, int j, long long flat, T* u, T*) { load(e, i, j, flat, u); },
        [&](int, int, int, long long, const T*, const T*) {}, store);
}

// apply_range with the input split in two: load(e,i,j,flat,u,aux) computes
// the staged inputs u and per-node values aux without writing global memory,
// so the loads of several nodes overlap; post(e,i,j,flat,u,aux) then does the
// caller's global stores for the node (aux is parked in the flux area, free
// until the flux phase).
template <int N, typename T, int OP, bool POST, class Load, class Post, class Store>
__device__ __forceinline__ void apply_range_post(T* sm, int kmax, const Fac<T>& fac,
                                                 const T* __restrict__ pot, T alpha, int e0, int ne,
                                                 Load&& load, Post&& post, Store&& store)
{
    constexpr int NN = N * N;
    constexpr int NC = op_nc<OP>();
    const int total = ne * NN;
    const int st = kmax * NN;
    const T* D = sm;
    T* su = sm + NN;
    T* sf1 = su + NC * st;
    T* sf2 = sf1 + NC * st;
    // 1. inputs of the whole range
#pragma unroll 4
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int le = t / NN;
        const int node = t - le * NN;
        const int e = e0 + le;
        T u[NC], aux[NC];
        load(e, node % N, node / N, (long long)e * NN + node, u, aux);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            su[c * st + t] = u[c];
            if (POST) sf1[c * st + t] = aux[c];
        }
    }
    if (POST) {
        for (int t = threadIdx.x; t < total; t += blockDim.x) {
            const int le = t / NN;
            const int node = t - le * NN;
            const int e = e0 + le;
            T u[NC], aux[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                u[c] = su[c * st + t];
                aux[c] = sf1[c * st + t];
            }
            post(e, node % N, node / N, (long long)e * NN + node, u, aux);
        }
    }
    __syncthreads();
    if (OP == OP_MASS) {
        for (int t = threadIdx.x; t < total; t += blockDim.x) {
            const int le = t / NN;
            const int node = t - le * NN;
            const int e = e0 + le;
            const long long flat = (long long)e * NN + node;
            T o[NC];
            o[0] = __ldg(fac.mass + flat) * su[t];
            store(e, node % N, node / N, flat, o);
        }
        __syncthreads();
        return;
    }
    // 2. contravariant fluxes
#pragma unroll 4
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int le = t / NN;
        const int node = t - le * NN;
        const int i = node % N, j = node / N;
        const long long flat = (long long)(e0 + le) * NN + node;
        const T g11 = __ldg(fac.g11 + flat), g12 = __ldg(fac.g12 + flat), g22 = __ldg(fac.g22 + flat);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T* uc = su + c * st + le * NN;
            T ur = T(0), us = T(0);
#pragma unroll
            for (int k = 0; k < N; ++k) {
                ur = fma(D[i * N + k], uc[k + j * N], ur);  // (D u)(i,j)
                us = fma(D[j * N + k], uc[i + k * N], us);  // (u D^T)(i,j)
            }
            sf1[c * st + t] = g11 * ur - g12 * us;
            sf2[c * st + t] = g22 * us - g12 * ur;
        }
    }
    __syncthreads();
    // 3. weak divergence + mass/potential terms
#pragma unroll 4
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int le = t / NN;
        const int node = t - le * NN;
        const int i = node % N, j = node / N;
        const int e = e0 + le;
        const long long flat = (long long)e * NN + node;
        T ms = T(0), pv = T(0);
        if (OP != OP_LAPLACE) ms = __ldg(fac.mass + flat);
        if (OP == OP_HELM || OP == OP_RES || OP == OP_F) pv = __ldg(pot + flat);
        T lap[NC], u[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T* f1 = sf1 + c * st + le * NN;
            const T* f2 = sf2 + c * st + le * NN;
            T a = T(0);
#pragma unroll
            for (int k = 0; k < N; ++k) a = fma(D[k * N + i], f1[k + j * N], a);
#pragma unroll
            for (int k = 0; k < N; ++k) a = fma(D[k * N + j], f2[i + k * N], a);
            lap[c] = a;
            u[c] = su[c * st + t];
        }
        T o[NC];
        if (OP == OP_LAPLACE) {
            o[0] = lap[0];
        } else if (OP == OP_HELM) {
            o[0] = lap[0] + (ms * pv) * u[0];
        } else if (OP == OP_RES) {
            const T mv = ms * pv;
            const T Lv = lap[NC - 1] + mv * u[NC - 1];
            const T Lu = lap[0] + mv * u[0];
            o[0] = ms * u[0] + alpha * Lv;
            o[NC - 1] = alpha * Lu - ms * u[NC - 1];
        } else {  // OP_F
            const T mv = ms * pv;
            o[0] = -(lap[NC - 1] + mv * u[NC - 1]);
            o[NC - 1] = -(lap[0] + mv * u[0]);
        }
        store(e, i, j, flat, o);
    }
    __syncthreads();
}

// ------------------------------------- element fast-diagonalisation pass
// Neumann-Neumann weight of an element-local copy: 1 / (number of elements
// sharing the node); 0 on the Dirichlet boundary
template <int N, typename T>
__device__ __forceinline__ T nn_weight(const DevMesh& m, const NodeInfo& ni, int e)
{
    if (ni.kind == 0) return T(1);
    const int c4 = ni.kind == 2 ? __ldg(m.corner_cnt4 + e) : 0;
    if (ni_boundary(ni)) return T(0);
    if (ni.kind == 1) return ni_lone(ni) ? T(1) : T(0.5);
    return T(1) / T((c4 >> (8 * ni.sc)) & 255);
}

template <typename T>
__device__ inline const T* fdm_s(const DevMesh& m);
template <>
__device__ inline const double* fdm_s<double>(const DevMesh& m) { return m.fdmS64; }
template <>
__device__ inline const float* fdm_s<float>(const DevMesh& m) { return m.fdmS32; }
template <typename T>
__device__ inline const T* fdm_l(const DevMesh& m);
template <>
__device__ inline const double* fdm_l<double>(const DevMesh& m) { return m.fdmL64; }
template <>
__device__ inline const float* fdm_l<float>(const DevMesh& m) { return m.fdmL32; }

// S and lambda of the mesh's degree into shared memory (every thread calls)
template <int N, typename T>
__device__ __forceinline__ void load_fdm_basis(T* S, T* lam, const DevMesh& m)
{
    const T* gs = fdm_s<T>(m);
    const T* gl = fdm_l<T>(m);
    for (int t = threadIdx.x; t < N * N; t += blockDim.x) S[t] = gs[t];
    for (int t = threadIdx.x; t < N; t += blockDim.x) lam[t] = gl[t];
}

// One block-wide pass of the element preconditioner over [e0, e0+ne),
// ne <= kmax, for the Schroedinger Res operator A = [M, aL; aL, -M]:
//   z_e = (S x S) diag(1 / sqrt(m^2 + a^2 l_kl^2)) (S x S)^T r_e     per plane,
//   l_kl = rx lambda_k + ry lambda_l,
// the inverse of |A_e| for the element's rectangle approximation (half
// widths ax, ay: mass m = ax ay, stiffness rx K (x) W + ry W (x) K with
// rx = ay/ax, ry = ax/ay), in the basis that diagonalises the 1-D GLL
// stiffness against the mass.  load(e,i,j,flat,u[NC]) supplies the
// (weighted) input, store(e,i,j,flat,z[NC]) receives the element result.
// Every thread of the block must call it.  S (S(i,k) at [i*N+k]) and lam
// are in shared memory; the staging area sm uses the apply's u/f1 regions
// (2 NC kmax N^2 values after the first N^2).
template <int N, typename T, int NC, bool POST, class Load, class Post, class Store>
__device__ __forceinline__ void fdm_range_post(T* sm, int kmax, const T* S, const T* lam, const DevMesh& m,
                                               T alpha, int e0, int ne, Load&& load, Post&& post, Store&& store);

template <int N, typename T, int NC, class Load, class Store>
__device__ __forceinline__ void fdm_range(T* sm, int kmax, const T* S, const T* lam, const DevMesh& m, T alpha,
                                          int e0, int ne, Load&& load, Store&& store)
{
    fdm_range_post<N, T, NC, false>(
        sm, kmax, S, lam, m, alpha, e0, ne,
        [&](int e, int i, int j, long long flat, T* u, T*) { load(e, i, j, flat, u); },
        [&](int, int, int, long long, const T*, const T*) {}, store);
}

// fdm_range with the input split as in apply_range_post (aux parked in the
// second staging area, free until the first contraction)
template <int N, typename T, int NC, bool POST, class Load, class Post, class Store>
__device__ __forceinline__ void fdm_range_post(T* sm, int kmax, const T* S, const T* lam, const DevMesh& m,
                                               T alpha, int e0, int ne, Load&& load, Post&& post, Store&& store)
{
    constexpr int NN = N * N;
    const int total = ne * NN;
    const int st = kmax * NN;
    T* su = sm + NN;
    T* stt = su + NC * st;
    // 0. inputs
#pragma unroll 4
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int le = t / NN;
        const int node = t - le * NN;
        const int e = e0 + le;
        T u[NC], aux[NC];
        load(e, node % N, node / N, (long long)e * NN + node, u, aux);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            su[c * st + t] = u[c];
            if (POST) stt[c * st + t] = aux[c];
        }
    }
    if (POST) {
        for (int t = threadIdx.x; t < total; t += blockDim.x) {
            const int le = t / NN;
            const int node = t - le * NN;
            const int e = e0 + le;
            T u[NC], aux[NC];
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                u[c] = su[c * st + t];
                aux[c] = stt[c * st + t];
            }
            post(e, node % N, node / N, (long long)e * NN + node, u, aux);
        }
    }
    __syncthreads();
    // 1. t(a,j) = sum_i S(i,a) u(i,j)
#pragma unroll 4
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int le = t / NN;
        const int node = t - le * NN;
        const int a = node % N, j = node / N;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T* uc = su + c * st + le * NN + j * N;
            T acc = T(0);
#pragma unroll
            for (int i = 0; i < N; ++i) acc = fma(S[i * N + a], uc[i], acc);
            stt[c * st + t] = acc;
        }
    }
    __syncthreads();
    // 2. u(a,b) = d(a,b) sum_j t(a,j) S(j,b)
#pragma unroll 4
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int le = t / NN;
        const int node = t - le * NN;
        const int a = node % N, b = node / N;
        const float4 g = __ldg(m.fdm_el + e0 + le);
        const T l = T(g.y) * lam[a] + T(g.z) * lam[b];
        const T mm = T(g.x);
        const T d = T(1) / sqrt(mm * mm + alpha * alpha * l * l);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T* tc = stt + c * st + le * NN + a;
            T acc = T(0);
#pragma unroll
            for (int j = 0; j < N; ++j) acc = fma(tc[j * N], S[j * N + b], acc);
            su[c * st + t] = d * acc;
        }
    }
    __syncthreads();
    // 3. t(i,b) = sum_a S(i,a) u(a,b)
#pragma unroll 4
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int le = t / NN;
        const int node = t - le * NN;
        const int i = node % N, b = node / N;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T* uc = su + c * st + le * NN + b * N;
            T acc = T(0);
#pragma unroll
            for (int a = 0; a < N; ++a) acc = fma(S[i * N + a], uc[a], acc);
            stt[c * st + t] = acc;
        }
    }
    __syncthreads();
    // 4. z(i,j) = sum_b t(i,b) S(j,b)
#pragma unroll 4
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int le = t / NN;
        const int node = t - le * NN;
        const int i = node % N, j = node / N;
        const int e = e0 + le;
        T z[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
            const T* tc = stt + c * st + le * NN + i;
            T acc = T(0);
#pragma unroll
            for (int b = 0; b < N; ++b) acc = fma(tc[b * N], S[j * N + b], acc);
            z[c] = acc;
        }
        store(e, i, j, (long long)e * NN + node, z);
    }
    __syncthreads();
}

// --------------------------------------------------------------- reductions
// block sum of a double, result returned to every thread (fixed order)
__device__ __forceinline__ double block_sum(double v, double* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        double s = lane < nw ? red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) red[32] = s;
    }
    __syncthreads();
    return red[32];
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier for cooperatively launched kernels.  One atomic per block:
// block 0 adds 2^31 - (G-1), every other block adds 1, so the counter's top
// bit flips exactly when the last block arrives and its low bits return to
// their start value (gs->count starts at 0).  Every wait is bounded: after
// timeout_ns the block records gs->err and returns false, so no block can spin
// forever.  Returns true when all blocks arrived.
__device__ __forceinline__ bool grid_barrier(GridSync* gs, long long timeout_ns)
{
    __syncthreads();
    if (!gs) return true;  // block-local solve (batched instances): the block barrier suffices
    if (threadIdx.x == 0) {
        const unsigned int inc = (blockIdx.x == 0) ? (0x80000000u - (gridDim.x - 1)) : 1u;
        volatile unsigned int* vc = &gs->count;
        volatile int* verr = &gs->err;
        __threadfence();
        const unsigned int old = atomicAdd(&gs->count, inc);
        if (((old ^ *vc) & 0x80000000u) == 0) {
            const unsigned long long t0 = global_ns();
            unsigned int polls = 0;
            while (((old ^ *vc) & 0x80000000u) == 0) {
                // the limit is checked on the first poll and every 64th after it
                if ((++polls & 63u) == 1) {
                    if (*verr) break;
                    if ((long long)(global_ns() - t0) > timeout_ns) {
                        atomicExch(&gs->err, 1);
                        break;
                    }
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *((volatile int*)&gs->err) == 0;
}

// all-reduce of one double across the grid: block sums to partials[slot][blk],
// barrier, then every block sums the partials in the same fixed order.
__device__ __forceinline__ double grid_sum(double v, double* partials, int slot, GridSync* gs,
                                           long long timeout_ns, double* red, bool& ok)
{
    const double bs = block_sum(v, red);
    const int G = gridDim.x;
    // same slot layout as grid_sum2 ([slot][2][grid]) so that consecutive
    // reductions (alternating slots) never share partial-sum words
    double* p = partials + (size_t)(2 * slot) * G;
    if (threadIdx.x == 0) p[blockIdx.x] = bs;
    ok = grid_barrier(gs, timeout_ns);
    if (threadIdx.x < 32) {
        double s = 0.0;
        for (int q = threadIdx.x; q < G; q += 32) s += __ldcg(p + q);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) red[33] = s;
    }
    __syncthreads();
    const double r = red[33];
    __syncthreads();
    return r;
}

// all-reduce of two doubles behind a single grid barrier; partials laid out
// [slot][2][grid] (the buffer holds 2 slots x 2 values x grid)
__device__ __forceinline__ void grid_sum2(double v0, double v1, double* partials, int slot, GridSync* gs,
                                          long long timeout_ns, double* red, bool& ok, double& r0, double& r1)
{
    const double b0 = block_sum(v0, red);
    const double b1 = block_sum(v1, red);
    const int G = gridDim.x;
    double* p0 = partials + (size_t)(slot * 2) * G;
    double* p1 = p0 + G;
    if (threadIdx.x == 0) {
        p0[blockIdx.x] = b0;
        p1[blockIdx.x] = b1;
    }
    ok = grid_barrier(gs, timeout_ns);
    if (threadIdx.x < 32) {
        double s0 = 0.0, s1 = 0.0;
        for (int q = threadIdx.x; q < G; q += 32) {
            s0 += __ldcg(p0 + q);
            s1 += __ldcg(p1 + q);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        }
        if (threadIdx.x == 0) {
            red[33] = s0;
            red[32] = s1;
        }
    }
    __syncthreads();
    r0 = red[33];
    r1 = red[32];
    __syncthreads();
}

}  // namespace semgb
