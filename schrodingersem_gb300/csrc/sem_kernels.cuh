// Kernel templates and their launchers.  Included by sem_inst.cu, which
// instantiates them for a list of polynomial degrees.
#pragma once
#include <cuda_runtime.h>

#include <cfloat>
#include <limits>

#include "sem_device.cuh"

namespace semgb {

// ------------------------------------------------------------ standalone ops

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

// ------------------------------------------------------ persistent MINRES
// include/minres.hpp:19-107 (identity preconditioner) as one cooperative
// kernel.  Lanczos vectors are kept in the continuous format (every copy of
// a shared node holds the assembled value, boundary zero) so the operator
// needs no gather; dots weight owner copies only, which makes them equal to
// the reference's masked-vector dots.  Per iteration: two grid barriers.
//   Phase B_i:   Av = DSS(Y)/beta_i; y = Av - (beta_i/beta_{i-1}) r1;
//                alpha_i = v.y;  pending w_{i-1}/x update
//   Phase A_i+1: y -= (alpha_i/beta_i) r2; beta_{i+1} = |y|; Y = A_local(y)
// The x update is applied to owner copies only, reproducing x += phi*w with
// the reference's masked w.
template <int N, typename T, int OP>
__global__ void __launch_bounds__(geo_tpb(N))
    k_minres(DevMesh m, SolveArgs a, KrylovWork<T> w)
{
    constexpr int NN = N * N;
    constexpr int K = geo_k(N);
    constexpr int NC = op_nc<OP>();
    __shared__ ApplySmem<N, T, OP> s;
    __shared__ double red[34];
    load_dmat(s, m);
    __syncthreads();
    const Fac<T> fac = fac_of<T>(m);
    const long long n = m.n;
    const T* pot = (const T*)a.pot;
    const T alpha = (T)a.alpha;
    const T* bp[2] = {(const T*)a.b[0], (const T*)a.b[1]};
    T* xp[2] = {(T*)a.x[0], (T*)a.x[1]};
    const int G = gridDim.x;
    const int eb = (int)((long long)blockIdx.x * m.E / G);
    const int ee = (int)((long long)(blockIdx.x + 1) * m.E / G);
    const long long nb = (long long)eb * NN, ne = (long long)ee * NN;
    int slot = 0;
    bool ok = true;
    T* L[3] = {w.L[0], w.L[1], w.L[2]};
    T* W[3] = {w.W[0], w.W[1], w.W[2]};
    int ir1 = 0, ir2 = 1, iy = 2;
    int iw1 = 0, iw2 = 1, iw = 2;

    auto store_y = [&](T* Yb) {
        return [=](int, int, int, long long flat, const T* o) {
#pragma unroll
            for (int c = 0; c < NC; ++c) Yb[c * n + flat] = o[c];
        };
    };

    // P0: Y[1] = A_local(unmask(x0))
    if (!a.x_is_zero) {
        for (int e0 = eb; e0 < ee; e0 += K)
            apply_chunk<N, T, OP>(
                s, fac, pot, alpha, e0, ee,
                [&](int e, int i, int j, long long flat, T* u) {
                    const long long src = ni_gather_src(m, node_info<N>(m, e, i, j), e, flat);
#pragma unroll
                    for (int c = 0; c < NC; ++c) u[c] = xp[c][src];
                },
                store_y(w.Y[1]));
        ok = grid_barrier(a.sync, a.timeout_ns);
        if (!ok) return;
    }
    // P1: r = unmask(b) - DSS(Y[1]); |r|^2; W[0] = W[1] = 0; Y[0] = A_local(r)
    double part = 0.0;
    for (int e0 = eb; e0 < ee; e0 += K)
        apply_chunk<N, T, OP>(
            s, fac, pot, alpha, e0, ee,
            [&](int e, int i, int j, long long flat, T* u) {
                const NodeInfo ni = node_info<N>(m, e, i, j);
                const long long src = ni_gather_src(m, ni, e, flat);
                const bool own = ni_owner(ni);
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    T r = bp[c][src];
                    if (!a.x_is_zero) r = r - dss_value<N, T, DSS_CONT>(m, w.Y[1] + c * n, ni, e, flat);
                    L[ir2][c * n + flat] = r;
                    W[iw1][c * n + flat] = T(0);
                    W[iw2][c * n + flat] = T(0);
                    u[c] = r;
                    if (own) part = fma((double)r, (double)r, part);
                }
            },
            store_y(w.Y[0]));
    const double bb = grid_sum(part, w.partials, slot, a.sync, a.timeout_ns, red, ok);
    slot ^= 1;
    if (!ok) return;

    const double eps_mach = (double)std::numeric_limits<T>::epsilon();
    const double bnorm = sqrt(bb);
    double beta = bnorm, beta_old = 0.0, phibar = bnorm, cs = -1.0, sn = 0.0, dbar = 0.0, eps = 0.0;
    double pg = 0.0, peps = 0.0, pdelta = 0.0, pphi = 0.0, pinvb = 0.0;
    bool pending = false, conv = false;
    int it = 1;
    if (a.maxit >= 1) {
        for (;;) {
            // ---- Phase B_it
            const T inv_b = (T)(1.0 / beta);
            const T c1 = (T)(it >= 2 ? beta / beta_old : 0.0);
            const T* Ycur = w.Y[(it - 1) & 1];
            double s1 = 0.0;
            for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
                const int e = (int)(idx / NN);
                const int node = (int)(idx - (long long)e * NN);
                const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
                const bool own = ni_owner(ni);
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    const long long q = c * n + idx;
                    const T av = dss_value<N, T, DSS_CONT>(m, Ycur + c * n, ni, e, idx) * inv_b;
                    T y3 = av;
                    T r1v = T(0);
                    if (it >= 2) {
                        r1v = L[ir1][q];
                        y3 = av - c1 * r1v;
                    }
                    const T vv = inv_b * L[ir2][q];
                    if (own) s1 = fma((double)vv, (double)y3, s1);
                    L[iy][q] = y3;
                    if (pending) {
                        const T vprev = (T)pinvb * r1v;
                        const T wn = (T)pg * ((vprev - (T)peps * W[iw1][q]) - (T)pdelta * W[iw2][q]);
                        W[iw][q] = wn;
                        if (own) xp[c][idx] += (T)pphi * wn;
                    }
                }
            }
            if (pending) {
                const int tmp = iw1;
                iw1 = iw2;
                iw2 = iw;
                iw = tmp;
                pending = false;
            }
            const double alpha_i = grid_sum(s1, w.partials, slot, a.sync, a.timeout_ns, red, ok);
            slot ^= 1;
            if (!ok) return;
            // ---- Phase A_it+1
            const T c2 = (T)(alpha_i / beta);
            double ss = 0.0;
            T* Ynext = w.Y[it & 1];
            for (int e0 = eb; e0 < ee; e0 += K)
                apply_chunk<N, T, OP>(
                    s, fac, pot, alpha, e0, ee,
                    [&](int e, int i, int j, long long flat, T* u) {
                        const bool own = ni_owner(node_info<N>(m, e, i, j));
#pragma unroll
                        for (int c = 0; c < NC; ++c) {
                            const long long q = c * n + flat;
                            const T y5 = L[iy][q] - c2 * L[ir2][q];
                            L[iy][q] = y5;
                            u[c] = y5;
                            if (own) ss = fma((double)y5, (double)y5, ss);
                        }
                    },
                    store_y(Ynext));
            const double bnew2 = grid_sum(ss, w.partials, slot, a.sync, a.timeout_ns, red, ok);
            slot ^= 1;
            if (!ok) return;
            const double beta_new = sqrt(bnew2);
            {
                const int tmp = ir1;
                ir1 = ir2;
                ir2 = iy;
                iy = tmp;
            }
            // ---- Givens rotation of iteration it (minres.hpp:65-84)
            const double eps_old = eps;
            const double delta = cs * dbar + sn * alpha_i;
            const double gbar = sn * dbar - cs * alpha_i;
            eps = sn * beta_new;
            dbar = -cs * beta_new;
            double gamma = sqrt(gbar * gbar + beta_new * beta_new);
            if (gamma < eps_mach) gamma = eps_mach;
            cs = gbar / gamma;
            sn = beta_new / gamma;
            const double phi = cs * phibar;
            phibar *= sn;
            pending = true;
            pg = 1.0 / gamma;
            peps = eps_old;
            pdelta = delta;
            pphi = phi;
            pinvb = 1.0 / beta;
            beta_old = beta;
            beta = beta_new;
            conv = phibar < a.tol * bnorm + a.tol;  // minres.hpp:92
            if (conv || it == a.maxit) break;
            ++it;
        }
        // ---- Phase F: w/x update of the last iteration
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
            const int e = (int)(idx / NN);
            const int node = (int)(idx - (long long)e * NN);
            const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
            if (!ni_owner(ni)) continue;
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const long long q = c * n + idx;
                const T vprev = (T)pinvb * L[ir1][q];
                const T wn = (T)pg * ((vprev - (T)peps * W[iw1][q]) - (T)pdelta * W[iw2][q]);
                xp[c][idx] += (T)pphi * wn;
            }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->success = conv ? 1 : 0;
        a.out->n_iter = conv ? it : (a.maxit >= 1 ? a.maxit + 1 : 1);
        a.out->residual = phibar;
        a.out->status = 0;
    }
}

// --------------------------------------------------------- persistent PCG
// include/pcg.hpp:59-97 with the identity preconditioner.  Vectors r, p in
// the continuous format; three grid barriers per iteration.
template <int N, typename T>
__global__ void __launch_bounds__(geo_tpb(N))
    k_pcg(DevMesh m, SolveArgs a, KrylovWork<T> w)
{
    constexpr int NN = N * N;
    constexpr int K = geo_k(N);
    __shared__ ApplySmem<N, T, OP_LAPLACE> s;
    __shared__ double red[34];
    load_dmat(s, m);
    __syncthreads();
    const Fac<T> fac = fac_of<T>(m);
    const T* b = (const T*)a.b[0];
    T* x = (T*)a.x[0];
    T* R = w.L[0];
    T* Pv = w.L[1];
    const int G = gridDim.x;
    const int eb = (int)((long long)blockIdx.x * m.E / G);
    const int ee = (int)((long long)(blockIdx.x + 1) * m.E / G);
    const long long nb = (long long)eb * NN, ne = (long long)ee * NN;
    int slot = 0;
    bool ok = true;
    auto store_y = [&](T* Yb) {
        return [=](int, int, int, long long flat, const T* o) { Yb[flat] = o[0]; };
    };
    if (!a.x_is_zero) {
        for (int e0 = eb; e0 < ee; e0 += K)
            apply_chunk<N, T, OP_LAPLACE>(
                s, fac, (const T*)nullptr, T(0), e0, ee,
                [&](int e, int i, int j, long long flat, T* u) {
                    u[0] = x[ni_gather_src(m, node_info<N>(m, e, i, j), e, flat)];
                },
                store_y(w.Y[1]));
        ok = grid_barrier(a.sync, a.timeout_ns);
        if (!ok) return;
    }
    double pb = 0.0, pr = 0.0;
    for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
        const T bv = b[ni_gather_src(m, ni, e, idx)];
        T r = bv;
        if (!a.x_is_zero) r = bv - dss_value<N, T, DSS_CONT>(m, w.Y[1], ni, e, idx);
        R[idx] = r;
        if (ni_owner(ni)) {
            pb = fma((double)bv, (double)bv, pb);
            pr = fma((double)r, (double)r, pr);
        }
    }
    const double bb = grid_sum(pb, w.partials, slot, a.sync, a.timeout_ns, red, ok);
    slot ^= 1;
    if (!ok) return;
    double rho = grid_sum(pr, w.partials, slot, a.sync, a.timeout_ns, red, ok);
    slot ^= 1;
    if (!ok) return;
    const double bnorm = sqrt(bb);
    double rho_prev = 0.0;
    bool conv = false;
    int it = 0;
    for (it = 0; it < a.maxit; ++it) {
        const T beta = (T)(it == 0 ? 0.0 : rho / rho_prev);
        for (int e0 = eb; e0 < ee; e0 += K)
            apply_chunk<N, T, OP_LAPLACE>(
                s, fac, (const T*)nullptr, T(0), e0, ee,
                [&](int, int, int, long long flat, T* u) {
                    const T pv = (it == 0) ? R[flat] : R[flat] + beta * Pv[flat];
                    Pv[flat] = pv;
                    u[0] = pv;
                },
                store_y(w.Y[0]));
        double pap = 0.0;
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
            const int e = (int)(idx / NN);
            const int node = (int)(idx - (long long)e * NN);
            const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
            if (ni_owner(ni))
                pap = fma((double)Pv[idx], (double)dss_value<N, T, DSS_CONT>(m, w.Y[0], ni, e, idx), pap);
        }
        const double pAp = grid_sum(pap, w.partials, slot, a.sync, a.timeout_ns, red, ok);
        slot ^= 1;
        if (!ok) return;
        const T al = (T)(rho / pAp);
        double prr = 0.0;
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
            const int e = (int)(idx / NN);
            const int node = (int)(idx - (long long)e * NN);
            const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
            const bool own = ni_owner(ni);
            const T ap = dss_value<N, T, DSS_CONT>(m, w.Y[0], ni, e, idx);
            if (own) x[idx] += al * Pv[idx];
            const T r = R[idx] - al * ap;
            R[idx] = r;
            if (own) prr = fma((double)r, (double)r, prr);
        }
        rho_prev = rho;
        conv = sqrt(rho) < a.tol * bnorm;  // pcg.hpp:84, rho of this iteration's start
        if (conv) break;
        rho = grid_sum(prr, w.partials, slot, a.sync, a.timeout_ns, red, ok);
        slot ^= 1;
        if (!ok) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->success = conv ? 1 : 0;
        a.out->n_iter = it;
        a.out->residual = sqrt(rho_prev);  // rho of the last iteration's start (pcg.hpp:93)
        a.out->status = 0;
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
cudaError_t launch_dss(const DevMesh& m, bool fp32, int mode, double scale, const void* y,
                       void* out, cudaStream_t st)
{
    const int tpb = 256;
    const int grid = grid_for(m.n, tpb);
#define SEM_DSS_CASE(T)                                                                            \
    switch (mode) {                                                                                \
        case DSS_SUM: k_dss<N, T, DSS_SUM><<<grid, tpb, 0, st>>>(m, (const T*)y, (T*)out, (T)scale); break; \
        case DSS_MASK: k_dss<N, T, DSS_MASK><<<grid, tpb, 0, st>>>(m, (const T*)y, (T*)out, (T)scale); break; \
        default: k_dss<N, T, DSS_CONT><<<grid, tpb, 0, st>>>(m, (const T*)y, (T*)out, (T)scale); break; \
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

template <int N, typename Kern>
static int coop_grid(Kern kern, int sms)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, geo_tpb(N), 0) != cudaSuccess)
        return 0;
    return per_sm * sms;
}

template <int N>
int solver_grid(int op, int nc, int sms)
{
    (void)nc;
    switch (op) {
        case OP_RES: return coop_grid<N>(k_minres<N, double, OP_RES>, sms);
        case OP_HELM: return coop_grid<N>(k_minres<N, double, OP_HELM>, sms);
        case OP_LAPLACE: return coop_grid<N>(k_pcg<N, double>, sms);
        default: return 0;
    }
}

template <int N>
cudaError_t launch_minres(const DevMesh& m, const SolveArgs& a, const KrylovWork<double>& w,
                          int grid, cudaStream_t st)
{
    DevMesh mm = m;
    SolveArgs aa = a;
    KrylovWork<double> ww = w;
    void* args[] = {&mm, &aa, &ww};
    const void* fn = (a.op == OP_RES) ? (const void*)k_minres<N, double, OP_RES>
                                      : (const void*)k_minres<N, double, OP_HELM>;
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(geo_tpb(N)), args, 0, st);
}

template <int N>
cudaError_t launch_pcg(const DevMesh& m, const SolveArgs& a, const KrylovWork<double>& w,
                       int grid, cudaStream_t st)
{
    DevMesh mm = m;
    SolveArgs aa = a;
    KrylovWork<double> ww = w;
    void* args[] = {&mm, &aa, &ww};
    return cudaLaunchCooperativeKernel((const void*)k_pcg<N, double>, dim3(grid), dim3(geo_tpb(N)),
                                       args, 0, st);
}

}  // namespace semgb

#define SEM_INSTANTIATE(NV)                                                                          \
    namespace semgb {                                                                                \
    template cudaError_t launch_apply<NV>(const DevMesh&, int, bool, const void*, double,            \
                                          const void*, const void*, void*, void*, bool,              \
                                          cudaStream_t);                                             \
    template cudaError_t launch_dss<NV>(const DevMesh&, bool, int, double, const void*, void*,       \
                                        cudaStream_t);                                               \
    template cudaError_t launch_unmask<NV>(const DevMesh&, bool, void*, cudaStream_t);               \
    template cudaError_t launch_mask<NV>(const DevMesh&, bool, void*, cudaStream_t);                 \
    template cudaError_t launch_dot<NV>(const DevMesh&, const double*, const double*, double*, int,  \
                                        int*, cudaStream_t);                                         \
    template cudaError_t launch_combo_f<NV>(const DevMesh&, const double*, const double*,            \
                                            const ZList&, double*, cudaStream_t);                    \
    template cudaError_t launch_update<NV>(const DevMesh&, const double*, const ZList&, double*,     \
                                           cudaStream_t);                                            \
    template cudaError_t launch_minres<NV>(const DevMesh&, const SolveArgs&,                         \
                                           const KrylovWork<double>&, int, cudaStream_t);            \
    template cudaError_t launch_pcg<NV>(const DevMesh&, const SolveArgs&, const KrylovWork<double>&, \
                                        int, cudaStream_t);                                          \
    template int solver_grid<NV>(int, int, int);                                                     \
    }
