// Persistent (cooperative) Krylov solvers: MINRES (FP64 or FP32), PCG, and
// FP64 iterative refinement around an FP32 inner MINRES.  One block per SM,
// SOLVER_TPB threads; each block owns a contiguous element range and stages
// up to kmax of its elements per pass in dynamic shared memory
// (apply_range).  Grid-wide phases are separated by bounded grid barriers.
//
// Scalar recurrences (Givens rotations, step lengths, stopping tests) run in
// FP64 on one thread per block and are broadcast through shared memory, with
// T-typed copies of the per-pass coefficients: GB300's FP64 pipe is 1/58 of
// FP32, so redundant per-thread scalar FP64 code would dominate small passes.
#pragma once
#include <cuda_runtime.h>

#include <cfloat>
#include <limits>

#include "sem_device.cuh"

namespace semgb {

constexpr int SOLVER_TPB = 512;

struct MinresOut {
    int it;
    double phibar;
    bool conv;
};

// block sum of per-thread T partials: warp shuffles in T, then FP64 across
// warps (fixed order); result returned to every thread
template <typename T>
__device__ __forceinline__ double block_sum_t(T v, double* red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = (double)v;
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

// grid all-reduce of up to two T partials (one barrier); see grid_sum2
template <typename T>
__device__ __forceinline__ void grid_sum2_t(T v0, T v1, double* partials, int slot, GridSync* gs, long long tmo,
                                            double* red, bool& ok, double& r0, double& r1)
{
    const double b0 = block_sum_t<T>(v0, red);
    const double b1 = block_sum_t<T>(v1, red);
    if (!gs) {  // block-local solve: the block sums are the sums
        ok = true;
        r0 = b0;
        r1 = b1;
        return;
    }
    const int G = gridDim.x;
    double* p0 = partials + (size_t)(slot * 2) * G;
    double* p1 = p0 + G;
    if (threadIdx.x == 0) {
        p0[blockIdx.x] = b0;
        p1[blockIdx.x] = b1;
    }
    ok = grid_barrier(gs, tmo);
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

// MINRES scalar state (minres.hpp:28-40, 65-84), shared memory, thread 0 only
template <typename T>
struct MinresScal {
    double bnorm, beta, beta_old, phibar, cs, sn, dbar, eps, inv_beta;
    double pg, peps, pdelta, pphi, pinvb, alpha_i;
    int pending, conv, stop;
    // coefficients of the next vector pass, in T
    T inv_b, c1, c2, cq, tpg, tpeps, tpdelta, tpphi, tpinvb;
};

template <typename T>
__device__ __forceinline__ void scal_init(MinresScal<T>& sc, double bnorm, double beta1)
{
    sc.bnorm = bnorm;
    sc.beta = beta1;
    sc.inv_beta = 1.0 / beta1;
    sc.beta_old = 0.0;
    sc.phibar = beta1;
    sc.cs = -1.0;
    sc.sn = 0.0;
    sc.dbar = 0.0;
    sc.eps = 0.0;
    sc.pg = sc.peps = sc.pdelta = sc.pphi = sc.pinvb = sc.alpha_i = 0.0;
    sc.pending = 0;
    sc.conv = 0;
    sc.stop = 0;
}

// coefficients of pass `it` (Phase B / fused pass)
template <typename T>
__device__ __forceinline__ void scal_publish(MinresScal<T>& sc, int it, double cq)
{
    sc.inv_b = (T)(1.0 / sc.beta);
    sc.c1 = (T)(it >= 2 ? sc.beta / sc.beta_old : 0.0);
    sc.cq = (T)cq;
    sc.tpg = (T)sc.pg;
    sc.tpeps = (T)sc.peps;
    sc.tpdelta = (T)sc.pdelta;
    sc.tpphi = (T)sc.pphi;
    sc.tpinvb = (T)sc.pinvb;
}

// Givens rotation of one iteration (minres.hpp:65-92)
template <typename T>
__device__ __forceinline__ void scal_givens(MinresScal<T>& sc, double alpha_i, double beta_new, double eps_mach,
                                            double tol_rel, double tol_abs)
{
    const double eps_old = sc.eps;
    const double delta = sc.cs * sc.dbar + sc.sn * alpha_i;
    const double gbar = sc.sn * sc.dbar - sc.cs * alpha_i;
    sc.eps = sc.sn * beta_new;
    sc.dbar = -sc.cs * beta_new;
    double gamma = sqrt(gbar * gbar + beta_new * beta_new);
    if (gamma < eps_mach) gamma = eps_mach;
    sc.cs = gbar / gamma;
    sc.sn = beta_new / gamma;
    const double phi = sc.cs * sc.phibar;
    sc.phibar *= sc.sn;
    sc.pending = 1;
    sc.pg = 1.0 / gamma;
    sc.peps = eps_old;
    sc.pdelta = delta;
    sc.pphi = phi;
    sc.pinvb = 1.0 / sc.beta;
    sc.beta_old = sc.beta;
    sc.beta = beta_new;
    sc.conv = sc.phibar < tol_rel * sc.bnorm + tol_abs;  // minres.hpp:92
}

// scal_givens + scal_publish of one iteration (it_next >= 2) for the FP32
// inner solver, with the square roots and reciprocals taken from two FP64
// reciprocal square roots: on one thread, GB300's FP64 division and square
// root are long dependent sequences on the critical path of every iteration.
template <typename T>
__device__ __forceinline__ void scal_step_rsqrt(MinresScal<T>& sc, double alpha_i, double bnew2, double eps_mach,
                                                double tol_rel, double tol_abs)
{
    const double inv_beta_new = bnew2 > 0.0 ? rsqrt(bnew2) : 1.0 / bnew2;
    const double beta_new = bnew2 > 0.0 ? bnew2 * inv_beta_new : 0.0;
    const double eps_old = sc.eps;
    const double delta = sc.cs * sc.dbar + sc.sn * alpha_i;
    const double gbar = sc.sn * sc.dbar - sc.cs * alpha_i;
    sc.eps = sc.sn * beta_new;
    sc.dbar = -sc.cs * beta_new;
    const double g2 = gbar * gbar + beta_new * beta_new;
    double ig = rsqrt(g2), gamma = g2 * ig;
    if (!(gamma >= eps_mach)) {
        gamma = eps_mach;
        ig = 1.0 / eps_mach;
    }
    sc.cs = gbar * ig;
    sc.sn = beta_new * ig;
    const double phi = sc.cs * sc.phibar;
    sc.phibar *= sc.sn;
    sc.pending = 1;
    sc.pg = ig;
    sc.peps = eps_old;
    sc.pdelta = delta;
    sc.pphi = phi;
    sc.pinvb = sc.inv_beta;
    const double c1 = beta_new * sc.inv_beta;
    sc.beta_old = sc.beta;
    sc.beta = beta_new;
    sc.inv_beta = inv_beta_new;
    sc.conv = sc.phibar < tol_rel * sc.bnorm + tol_abs;  // minres.hpp:92
    sc.inv_b = (T)inv_beta_new;
    sc.c1 = (T)c1;
    sc.cq = T(0);
    sc.tpg = (T)sc.pg;
    sc.tpeps = (T)sc.peps;
    sc.tpdelta = (T)sc.pdelta;
    sc.tpphi = (T)sc.pphi;
    sc.tpinvb = (T)sc.pinvb;
}

// One node of MINRES Phase B: Av = DSS(Y)/beta, y = Av - c1 r1, the
// alpha partial v.y, and (pending) the w / x update of the previous
// iteration.  The vectors arrive as restrict pointers (distinct buffers), so
// that once inlined into an unrolled node loop the loads of the next node
// can be issued before the stores of this one.
template <int N, typename T, int NC, int PRE>
__device__ __forceinline__ void phase_b_node(const DevMesh& m, long long n, long long idx, int it, bool pending,
                                             T inv_b, T c1, T tpg, T tpeps, T tpdelta, T tpphi, T tpinvb,
                                             const T* __restrict__ Ycur, const T* __restrict__ Lr1,
                                             const T* __restrict__ Zc, const T* __restrict__ Zq,
                                             const T* __restrict__ W1, const T* __restrict__ W2,
                                             const T* __restrict__ pinv, T* __restrict__ Ly, T* __restrict__ Wn,
                                             T* __restrict__ x0, T* __restrict__ x1, T& s1)
{
    constexpr int NN = N * N;
    const int e = (int)(idx / NN);
    const int node = (int)(idx - (long long)e * NN);
    const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
    const bool own = ni_owner(ni);
    const T pv = PRE == 1 ? pinv[idx] : T(1);
    T av[NC], r1v[NC], zc[NC], zp[NC], w1v[NC], w2v[NC], xv[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const long long q = c * n + idx;
        av[c] = dss_value<N, T, DSS_CONT>(m, Ycur + c * n, ni, e, idx);
        r1v[c] = it >= 2 ? Lr1[q] : T(0);
        zc[c] = Zc[q];
        if (pending) {
            zp[c] = PRE == 2 ? Zq[q] : T(0);
            w1v[c] = W1[q];
            w2v[c] = W2[q];
            if (own) xv[c] = (c == 0 ? x0 : x1)[idx];
        }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const long long q = c * n + idx;
        const T a = av[c] * inv_b;
        const T y3 = it >= 2 ? a - c1 * r1v[c] : a;
        const T vv = inv_b * (PRE == 1 ? pv * zc[c] : zc[c]);
        if (own) s1 = fma(vv, y3, s1);
        Ly[q] = y3;
        if (pending) {
            const T vprev = tpinvb * (PRE == 2 ? zp[c] : PRE == 1 ? pv * r1v[c] : r1v[c]);
            const T wn = tpg * ((vprev - tpeps * w1v[c]) - tpdelta * w2v[c]);
            Wn[q] = wn;
            if (own) (c == 0 ? x0 : x1)[idx] = xv[c] + tpphi * wn;
        }
    }
}

// include/minres.hpp:19-107 inside a cooperative kernel.  Lanczos vectors
// are kept in the continuous format (every copy of a shared node holds the
// assembled value, boundary zero) so the operator needs no gather; dots
// weight owner copies only, which makes them equal to the reference's
// masked-vector dots.  Per iteration two grid barriers:
//   Phase B_i:   Av = DSS(Y)/beta_i; y = Av - (beta_i/beta_{i-1}) r1;
//                alpha_i = v.y;  pending w_{i-1} / x update
//   Phase A_i+1: y -= (alpha_i/beta_i) r2; z = P^-1 y; beta_{i+1}^2 = y.z;
//                Y = A_local(z)
// x is updated on owner copies only, reproducing x += phi*w with the
// reference's masked w.  Stops when phibar < tol_rel*|r0| + tol_abs.  With
// PRE a diagonal preconditioner P^-1 (continuous format) is applied in the
// Paige-Saunders form beta = sqrt(r2 . P^-1 r2).
// rhs(ni, e, flat, c) gives the initial residual (continuous format) at a
// node.  Returns false when a grid barrier timed out.
template <int N, typename T, int OP, int PRE, class Rhs>
__device__ __forceinline__ bool minres_core(T* sm, int kmax, double* red, MinresScal<T>& sc, const DevMesh& m,
                                            const T* pot, T alpha, int eb, int ee,
                                            const KrylovWork<T>& w, GridSync* gs, long long tmo,
                                            int& slot, Rhs&& rhs, T* const* xp, int maxit,
                                            double tol_rel, double tol_abs, MinresOut& res,
                                            const T* __restrict__ pinv, const T* fS = nullptr,
                                            const T* fL = nullptr)
{
    constexpr int NN = N * N;
    constexpr int NC = op_nc<OP>();
    const Fac<T> fac = fac_of<T>(m);
    const long long n = m.n;
    const long long nb = (long long)eb * NN, ne = (long long)ee * NN;
    const double eps_mach = (double)std::numeric_limits<T>::epsilon();
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
    // P1: r; |r|^2 and r.z (z = P^-1 r); W[0] = W[1] = 0; Y[0] = A_local(z)
    T part = T(0), partz = T(0);
    if constexpr (PRE == 2) {
        // element preconditioner: weighted local solves into Y[1], then
        // z = DSS (continuous) kept in Z[0]
        T* Zl = w.Y[1];
        for (int e0 = eb; e0 < ee; e0 += kmax)
            fdm_range<N, T, NC>(
                sm, kmax, fS, fL, m, alpha, e0, min(kmax, ee - e0),
                [&](int e, int i, int j, long long flat, T* u) {
                    const NodeInfo ni = node_info<N>(m, e, i, j);
                    const bool own = ni_owner(ni);
                    const T wt = nn_weight<N, T>(m, ni, e);
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        const T r = rhs(ni, e, flat, c);
                        L[ir2][c * n + flat] = r;
                        W[iw1][c * n + flat] = T(0);
                        W[iw2][c * n + flat] = T(0);
                        u[c] = wt * r;
                        if (own) part = fma(r, r, part);
                    }
                },
                [&](int e, int i, int j, long long flat, const T* z) {
                    const T wt = nn_weight<N, T>(m, node_info<N>(m, e, i, j), e);
#pragma unroll
                    for (int c = 0; c < NC; ++c) Zl[c * n + flat] = wt * z[c];
                });
        if (!grid_barrier(gs, tmo)) return false;
        for (int e0 = eb; e0 < ee; e0 += kmax)
            apply_range<N, T, OP>(
                sm, kmax, fac, pot, alpha, e0, min(kmax, ee - e0),
                [&](int e, int i, int j, long long flat, T* u) {
                    const NodeInfo ni = node_info<N>(m, e, i, j);
                    const bool own = ni_owner(ni);
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        const T z = dss_value<N, T, DSS_CONT>(m, Zl + c * n, ni, e, flat);
                        w.Z[0][c * n + flat] = z;
                        u[c] = z;
                        if (own) partz = fma(L[ir2][c * n + flat], z, partz);
                    }
                },
                store_y(w.Y[0]));
    } else {
        for (int e0 = eb; e0 < ee; e0 += kmax)
            apply_range<N, T, OP>(
                sm, kmax, fac, pot, alpha, e0, min(kmax, ee - e0),
                [&](int e, int i, int j, long long flat, T* u) {
                    const NodeInfo ni = node_info<N>(m, e, i, j);
                    const bool own = ni_owner(ni);
                    const T pv = PRE == 1 ? pinv[flat] : T(1);
#pragma unroll
                    for (int c = 0; c < NC; ++c) {
                        const T r = rhs(ni, e, flat, c);
                        L[ir2][c * n + flat] = r;
                        W[iw1][c * n + flat] = T(0);
                        W[iw2][c * n + flat] = T(0);
                        const T z = PRE == 1 ? pv * r : r;
                        u[c] = z;
                        if (own) {
                            part = fma(r, r, part);
                            partz = fma(r, z, partz);
                        }
                    }
                },
                store_y(w.Y[0]));
    }
    double bb = 0.0, bz = 0.0;
    grid_sum2_t<T>(part, partz, w.partials, slot, gs, tmo, red, ok, bb, bz);
    slot ^= 1;
    if (!ok) return false;
    if (threadIdx.x == 0) {
        // minres.hpp:28,31; preconditioned runs measure the stop relative to
        // the preconditioned norm sqrt(r.P^-1 r) their phibar estimates
        scal_init(sc, PRE ? sqrt(bz) : sqrt(bb), sqrt(bz));
        scal_publish(sc, 1, 0.0);
    }
    __syncthreads();
    int it = 1;
    if (maxit >= 1) {
        for (;;) {
            // ---- Phase B_it
            const T inv_b = sc.inv_b, c1 = sc.c1;
            const bool pending = sc.pending != 0;
            const T tpg = sc.tpg, tpeps = sc.tpeps, tpdelta = sc.tpdelta, tpphi = sc.tpphi, tpinvb = sc.tpinvb;
            const T* Ycur = w.Y[(it - 1) & 1];
            T s1 = T(0);
            const T* Zc = PRE == 2 ? w.Z[(it - 1) & 1] : L[ir2];
            const T* Zq = PRE == 2 ? w.Z[it & 1] : nullptr;
            T* const x1 = NC == 2 ? xp[1] : nullptr;
#pragma unroll 2
            for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x)
                phase_b_node<N, T, NC, PRE>(m, n, idx, it, pending, inv_b, c1, tpg, tpeps, tpdelta, tpphi, tpinvb,
                                            Ycur, L[ir1], Zc, Zq, W[iw1], W[iw2], pinv, L[iy], W[iw], xp[0], x1,
                                            s1);
            if (pending) {
                const int tmp = iw1;
                iw1 = iw2;
                iw2 = iw;
                iw = tmp;
            }
            if constexpr (PRE == 2) {
                // local solves of y itself, ahead of alpha: the preconditioner
                // is linear, so P^-1 y5 = P^-1 y - (alpha/beta) z_it is formed
                // in Phase A without a barrier of its own (y of this block's
                // elements is complete after the block barrier)
                __syncthreads();
                for (int e0 = eb; e0 < ee; e0 += kmax)
                    fdm_range<N, T, NC>(
                        sm, kmax, fS, fL, m, alpha, e0, min(kmax, ee - e0),
                        [&](int e, int i, int j, long long flat, T* u) {
                            const T wt = nn_weight<N, T>(m, node_info<N>(m, e, i, j), e);
#pragma unroll
                            for (int c = 0; c < NC; ++c) u[c] = wt * L[iy][c * n + flat];
                        },
                        [&](int e, int i, int j, long long flat, const T* z) {
                            const T wt = nn_weight<N, T>(m, node_info<N>(m, e, i, j), e);
#pragma unroll
                            for (int c = 0; c < NC; ++c) w.Y3[c * n + flat] = wt * z[c];
                        });
            }
            double S1 = 0.0, dummy = 0.0;
            grid_sum2_t<T>(s1, T(0), w.partials, slot, gs, tmo, red, ok, S1, dummy);
            slot ^= 1;
            if (!ok) return false;
            if (threadIdx.x == 0) {
                sc.pending = 0;
                sc.alpha_i = S1;
                sc.c2 = (T)(S1 / sc.beta);
            }
            __syncthreads();
            // ---- Phase A_it+1
            const T c2 = sc.c2;
            T ss = T(0);
            T* Ynext = w.Y[it & 1];
            if constexpr (PRE == 2) {
                // z_{it+1} = DSS(local solves of y) - c2 z_it, y5 = y - c2 r2
                const T* Zc = w.Z[(it - 1) & 1];
                T* Zn = w.Z[it & 1];
                for (int e0 = eb; e0 < ee; e0 += kmax)
                    apply_range_post<N, T, OP, true>(
                        sm, kmax, fac, pot, alpha, e0, min(kmax, ee - e0),
                        [&](int e, int i, int j, long long flat, T* u, T* aux) {
                            const NodeInfo ni = node_info<N>(m, e, i, j);
#pragma unroll
                            for (int c = 0; c < NC; ++c) {
                                const long long q = c * n + flat;
                                u[c] = dss_value<N, T, DSS_CONT>(m, w.Y3 + c * n, ni, e, flat) - c2 * Zc[q];
                                aux[c] = L[iy][q] - c2 * L[ir2][q];
                            }
                        },
                        [&](int e, int i, int j, long long flat, const T* u, const T* aux) {
                            const bool own = ni_owner(node_info<N>(m, e, i, j));
#pragma unroll
                            for (int c = 0; c < NC; ++c) {
                                L[iy][c * n + flat] = aux[c];
                                Zn[c * n + flat] = u[c];
                                if (own) ss = fma(aux[c], u[c], ss);
                            }
                        },
                        store_y(Ynext));
            } else {
                for (int e0 = eb; e0 < ee; e0 += kmax)
                    apply_range_post<N, T, OP, true>(
                        sm, kmax, fac, pot, alpha, e0, min(kmax, ee - e0),
                        [&](int, int, int, long long flat, T* u, T* aux) {
                            const T pv = PRE == 1 ? pinv[flat] : T(1);
#pragma unroll
                            for (int c = 0; c < NC; ++c) {
                                const long long q = c * n + flat;
                                const T y5 = L[iy][q] - c2 * L[ir2][q];
                                aux[c] = y5;
                                u[c] = PRE == 1 ? pv * y5 : y5;  // y = precond(r2), minres.hpp:60
                            }
                        },
                        [&](int e, int i, int j, long long flat, const T* u, const T* aux) {
                            const bool own = ni_owner(node_info<N>(m, e, i, j));
#pragma unroll
                            for (int c = 0; c < NC; ++c) {
                                L[iy][c * n + flat] = aux[c];
                                if (own) ss = fma(aux[c], u[c], ss);
                            }
                        },
                        store_y(Ynext));
            }
            double bnew2 = 0.0;
            grid_sum2_t<T>(ss, T(0), w.partials, slot, gs, tmo, red, ok, bnew2, dummy);
            slot ^= 1;
            if (!ok) return false;
            {
                const int tmp = ir1;
                ir1 = ir2;
                ir2 = iy;
                iy = tmp;
            }
            if (threadIdx.x == 0) {
                if constexpr (sizeof(T) == 4) {
                    scal_step_rsqrt(sc, sc.alpha_i, bnew2, eps_mach, tol_rel, tol_abs);
                    sc.stop = sc.conv || it == maxit;
                } else {
                    scal_givens(sc, sc.alpha_i, sqrt(bnew2), eps_mach, tol_rel, tol_abs);
                    sc.stop = sc.conv || it == maxit;
                    scal_publish(sc, it + 1, 0.0);
                }
            }
            __syncthreads();
            if (sc.stop) break;
            ++it;
        }
        // ---- Phase F: w/x update of the last iteration
        const T tpg = sc.tpg, tpeps = sc.tpeps, tpdelta = sc.tpdelta, tpphi = sc.tpphi, tpinvb = sc.tpinvb;
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
            const int e = (int)(idx / NN);
            const int node = (int)(idx - (long long)e * NN);
            const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
            if (!ni_owner(ni)) continue;
            const T pv = PRE == 1 ? pinv[idx] : T(1);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const long long q = c * n + idx;
                const T vprev = tpinvb * (PRE == 2 ? w.Z[(it - 1) & 1][q] : PRE == 1 ? pv * L[ir1][q] : L[ir1][q]);
                const T wn = tpg * ((vprev - tpeps * W[iw1][q]) - tpdelta * W[iw2][q]);
                xp[c][idx] += tpphi * wn;
            }
        }
    }
    res.it = it;
    res.phibar = sc.phibar;
    res.conv = sc.conv != 0;
    __syncthreads();
    return true;
}

// Single-barrier variant of minres_core (same recurrences, Givens rotations
// and stopping test) for the Res operator in the FP32 inner solve.  The
// element operator is linear, so the next operator product is carried as
//   A z_{i+1} = DSS(A_local(P^-1 y_i)) - (alpha_i/beta_i) A z_i,
// with A_local(P^-1 y_i) computed in the same pass that forms y_i, and
//   beta_{i+1}^2 = y_i . P^-1 y_i - alpha_i^2
// comes out of the same reduction as alpha_i = z_i . y_i / beta_i.  The
// subtraction is benign for Res = [M, aL; aL, -M], whose spectrum is
// symmetric about zero (Lanczos alpha_i stay small against beta_i); it
// would cancel for one-sided spectra, which therefore use minres_core.
// Rounding in the recurred A z is not re-anchored: the FP64 refinement
// around the inner solve judges the true residual.
template <int N, typename T, int OP, bool PRE, class Rhs>
__device__ __forceinline__ bool minres_core_fused(T* sm, int kmax, double* red, MinresScal<T>& sc,
                                                  const DevMesh& m, const T* pot, T alpha, int eb, int ee,
                                                  const KrylovWork<T>& w, GridSync* gs, long long tmo,
                                                  int& slot, Rhs&& rhs, T* const* xp, int maxit,
                                                  double tol_rel, double tol_abs, MinresOut& res,
                                                  const T* __restrict__ pinv)
{
    constexpr int NN = N * N;
    constexpr int NC = op_nc<OP>();
    const Fac<T> fac = fac_of<T>(m);
    const long long n = m.n;
    const long long nb = (long long)eb * NN, ne = (long long)ee * NN;
    const double eps_mach = (double)std::numeric_limits<T>::epsilon();
    bool ok = true;
    T* Q[3] = {w.L[0], w.L[1], w.L[2]};  // q_i (= r2), q_{i-1} (= r1), free
    T* W[3] = {w.W[0], w.W[1], w.W[2]};
    T* TT[2] = {w.Y[0], w.Y[1]};         // element-local A_local(P^-1 y) ping-pong
    T* AZ = w.AZ;
    T* Y3 = w.Y3;
    int iq = 0, iq1 = 1, iqf = 2;
    int iw1 = 0, iw2 = 1, iw = 2;
    auto store_t = [&](T* Tb) {
        return [=](int, int, int, long long flat, const T* o) {
#pragma unroll
            for (int c = 0; c < NC; ++c) Tb[c * n + flat] = o[c];
        };
    };
    // P1: q_1 = r0, z_1 = P^-1 q_1; |r0|^2, q_1.z_1; W[0] = W[1] = 0; T[1] = A_local(z_1)
    T part = T(0), partz = T(0);
    for (int e0 = eb; e0 < ee; e0 += kmax)
        apply_range<N, T, OP>(
            sm, kmax, fac, pot, alpha, e0, min(kmax, ee - e0),
            [&](int e, int i, int j, long long flat, T* u) {
                const NodeInfo ni = node_info<N>(m, e, i, j);
                const bool own = ni_owner(ni);
                const T pv = PRE ? pinv[flat] : T(1);
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    const T r = rhs(ni, e, flat, c);
                    Q[iq][c * n + flat] = r;
                    W[iw1][c * n + flat] = T(0);
                    W[iw2][c * n + flat] = T(0);
                    const T z = PRE ? pv * r : r;
                    u[c] = z;
                    if (own) {
                        part = fma(r, r, part);
                        partz = fma(r, z, partz);
                    }
                }
            },
            store_t(TT[1]));
    double bb = 0.0, bz = 0.0;
    grid_sum2_t<T>(part, partz, w.partials, slot, gs, tmo, red, ok, bb, bz);
    slot ^= 1;
    if (!ok) return false;
    if (threadIdx.x == 0) {
        scal_init(sc, PRE ? sqrt(bz) : sqrt(bb), sqrt(bz));  // as minres_core
        scal_publish(sc, 1, 0.0);
    }
    __syncthreads();
    int it = 1;
    if (maxit >= 1) {
        for (;;) {
            const T inv_b = sc.inv_b, c1 = sc.c1, cq = sc.cq;
            const bool pending = sc.pending != 0;
            const T tpg = sc.tpg, tpeps = sc.tpeps, tpdelta = sc.tpdelta, tpphi = sc.tpphi, tpinvb = sc.tpinvb;
            const bool first = (it == 1);
            const T* Tin = TT[it & 1];  // A_local of the previous pass
            T* Tout = TT[(it + 1) & 1];
            T s1 = T(0), s2 = T(0);
            for (int e0 = eb; e0 < ee; e0 += kmax)
                apply_range<N, T, OP>(
                    sm, kmax, fac, pot, alpha, e0, min(kmax, ee - e0),
                    [&](int e, int i, int j, long long flat, T* u) {
                        const NodeInfo ni = node_info<N>(m, e, i, j);
                        const bool own = ni_owner(ni);
                        const T pv = PRE ? pinv[flat] : T(1);
#pragma unroll
                        for (int c = 0; c < NC; ++c) {
                            const long long q = c * n + flat;
                            const T tsum = dss_value<N, T, DSS_CONT>(m, Tin + c * n, ni, e, flat);
                            T qi, az, r1v = T(0);
                            if (first) {
                                qi = Q[iq][q];
                                az = tsum;
                            } else {
                                r1v = Q[iq1][q];
                                qi = Y3[q] - cq * r1v;  // q_i = y_{i-1} - (alpha/beta) q_{i-1}
                                az = tsum - cq * AZ[q];
                                Q[iq][q] = qi;
                            }
                            AZ[q] = az;
                            const T y = az * inv_b - c1 * r1v;
                            Y3[q] = y;
                            const T zi = PRE ? pv * qi : qi;
                            const T py = PRE ? pv * y : y;
                            if (own) {
                                s1 = fma(zi, y, s1);
                                s2 = fma(y, py, s2);
                            }
                            if (pending) {
                                const T vprev = tpinvb * (PRE ? pv * r1v : r1v);
                                const T wn = tpg * ((vprev - tpeps * W[iw1][q]) - tpdelta * W[iw2][q]);
                                W[iw][q] = wn;
                                if (own) xp[c][flat] += tpphi * wn;
                            }
                            u[c] = py;
                        }
                    },
                    store_t(Tout));
            if (pending) {
                const int tmp = iw1;
                iw1 = iw2;
                iw2 = iw;
                iw = tmp;
            }
            double S1 = 0.0, S2 = 0.0;
            grid_sum2_t<T>(s1, s2, w.partials, slot, gs, tmo, red, ok, S1, S2);
            slot ^= 1;
            if (!ok) return false;
            {
                const int tmp = iqf;  // the next pass writes q_{i+1} into the free slot
                iqf = iq1;
                iq1 = iq;
                iq = tmp;
            }
            if (threadIdx.x == 0) {
                const double alpha_i = S1 / sc.beta;
                double bnew2 = S2 - alpha_i * alpha_i;
                if (bnew2 < 0.0) bnew2 = 0.0;
                const double cnext = alpha_i / sc.beta;
                scal_givens(sc, alpha_i, sqrt(bnew2), eps_mach, tol_rel, tol_abs);
                sc.stop = sc.conv || it == maxit || sc.beta == 0.0;
                scal_publish(sc, it + 1, cnext);
            }
            __syncthreads();
            if (sc.stop) break;
            ++it;
        }
        // ---- final w/x update of the last iteration (v = P^-1 q_it / beta_it; q_it is Q[iq1])
        const T tpg = sc.tpg, tpeps = sc.tpeps, tpdelta = sc.tpdelta, tpphi = sc.tpphi, tpinvb = sc.tpinvb;
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
            const int e = (int)(idx / NN);
            const int node = (int)(idx - (long long)e * NN);
            const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
            if (!ni_owner(ni)) continue;
            const T pv = PRE ? pinv[idx] : T(1);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const long long q = c * n + idx;
                const T vprev = tpinvb * (PRE ? pv * Q[iq1][q] : Q[iq1][q]);
                const T wn = tpg * ((vprev - tpeps * W[iw1][q]) - tpdelta * W[iw2][q]);
                xp[c][idx] += tpphi * wn;
            }
        }
    }
    res.it = it;
    res.phibar = sc.phibar;
    res.conv = sc.conv != 0;
    __syncthreads();
    return true;
}

__device__ __forceinline__ void block_range(int E, int& eb, int& ee)
{
    const int G = gridDim.x;
    eb = (int)((long long)blockIdx.x * E / G);
    ee = (int)((long long)(blockIdx.x + 1) * E / G);
}

// ---------------------------------------------------------- plain MINRES
template <int N, typename T, int OP>
__global__ void __launch_bounds__(SOLVER_TPB, 1)
    k_minres(DevMesh m, SolveArgs a, KrylovWork<T> w)
{
    constexpr int NC = op_nc<OP>();
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[34];
    __shared__ MinresScal<T> sc;
    T* sm = (T*)smraw;
    load_dmat_raw<N, T>(sm, m);
    __syncthreads();
    const Fac<T> fac = fac_of<T>(m);
    const long long n = m.n;
    const T* pot = (const T*)a.pot;
    const T alpha = (T)a.alpha;
    const T* bp[2] = {(const T*)a.b[0], (const T*)a.b[1]};
    T* xp[2] = {(T*)a.x[0], (T*)a.x[1]};
    int eb, ee;
    block_range(m.E, eb, ee);
    const int kmax = a.kmax;
    int slot = 0;
    // P0: Y[1] = A_local(unmask(x0))
    if (!a.x_is_zero) {
        T* Y1 = w.Y[1];
        for (int e0 = eb; e0 < ee; e0 += kmax)
            apply_range<N, T, OP>(
                sm, kmax, fac, pot, alpha, e0, min(kmax, ee - e0),
                [&](int e, int i, int j, long long flat, T* u) {
                    const long long src = ni_gather_src(m, node_info<N>(m, e, i, j), e, flat);
#pragma unroll
                    for (int c = 0; c < NC; ++c) u[c] = xp[c][src];
                },
                [&](int, int, int, long long flat, const T* o) {
#pragma unroll
                    for (int c = 0; c < NC; ++c) Y1[c * n + flat] = o[c];
                });
        if (!grid_barrier(a.sync, a.timeout_ns)) return;
    }
    // r0 = unmask(b) - DSS(A_local(unmask(x0)))
    const bool xz = a.x_is_zero != 0;
    const T* Y1 = w.Y[1];
    auto rhs = [&](const NodeInfo& ni, int e, long long flat, int c) -> T {
        T r = bp[c][ni_gather_src(m, ni, e, flat)];
        if (!xz) r = r - dss_value<N, T, DSS_CONT>(m, Y1 + c * n, ni, e, flat);
        return r;
    };
    MinresOut r{};
    if (!minres_core<N, T, OP, 0>(sm, kmax, red, sc, m, pot, alpha, eb, ee, w, a.sync, a.timeout_ns, slot,
                                      rhs, xp, a.maxit, a.tol, a.tol, r, (const T*)nullptr))
        return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->success = r.conv ? 1 : 0;
        a.out->n_iter = r.conv ? r.it : (a.maxit >= 1 ? a.maxit + 1 : 1);
        a.out->residual = r.phibar;
        a.out->status = 0;
    }
}

// ------------------------------------------- mixed-precision refinement
// FP64 iterative refinement around an FP32 inner MINRES.  Each sweep:
// r = b - A x in FP64 (true residual, continuous format); stop when
// |r| < tol |r_0| + tol (for x_0 = 0 the reference's criterion minres.hpp:92
// with the true residual in place of the recursive estimate; with rel_to_b,
// |b| replaces |r_0|); else solve A d = r in FP32 to relative tolerance
// inner_tol and add d to x in FP64 on owner copies.
//
// The refinement itself is a device function over the element range
// [eb, ee): the cooperative kernel gives every block a slice of one mesh
// (grid barriers and grid reductions); the batched kernel gives one block a
// whole instance (a.sync == nullptr: block barriers and block reductions).
// Returns false when a wait timed out.  `leader` writes a.out.  LEAN
// compiles only the unpreconditioned and element-preconditioned inner
// iterations (the batched kernels).
template <int N, int OP, bool LEAN = false>
__device__ __forceinline__ bool mixed_solve(const DevMesh& m, const SolveArgs& a, const KrylovWork<float>& w,
                                            const MixedArgs& mx, int eb, int ee, bool leader,
                                            unsigned char* smraw, double* red, MinresScal<float>& sc,
                                            double* sweep_state, float* fdmS, float* fdmL)
{
    constexpr int NN = N * N;
    constexpr int NC = op_nc<OP>();
    double* sm64 = (double*)smraw;
    float* sm32 = (float*)smraw;
    const Fac<double> fac64 = fac_of<double>(m);
    const double* pot64 = (const double*)a.pot;
    const double* bp[2] = {(const double*)a.b[0], (const double*)a.b[1]};
    double* xp[2] = {(double*)a.x[0], (double*)a.x[1]};
    const long long nb = (long long)eb * NN, ne = (long long)ee * NN;
    const int kmax = a.kmax;
    int slot = 0;
    bool ok = true;
    int sweep = 0, inner_total = 0;
    bool conv = false;
    for (;;) {
        // ---- FP64 residual r = unmask(b) - DSS(A_local(unmask(x)))
        const bool applied = (sweep > 0) || !a.x_is_zero;
        if (applied) {
            load_dmat_raw<N, double>(sm64, m);
            __syncthreads();
            for (int e0 = eb; e0 < ee; e0 += kmax)
                apply_range<N, double, OP>(
                    sm64, kmax, fac64, pot64, a.alpha, e0, min(kmax, ee - e0),
                    [&](int e, int i, int j, long long flat, double* u) {
                        const long long src = ni_gather_src(m, node_info<N>(m, e, i, j), e, flat);
#pragma unroll
                        for (int c = 0; c < NC; ++c) u[c] = xp[c][src];
                    },
                    [&](int, int, int, long long flat, const double* o) {
#pragma unroll
                        for (int c = 0; c < NC; ++c) mx.Y64[c][flat] = o[c];
                    });
            if (!grid_barrier(a.sync, a.timeout_ns)) return false;
        }
        double part = 0.0, partb = 0.0;
        const bool want_b = (sweep == 0) && a.rel_to_b;
#pragma unroll 4
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
            const int e = (int)(idx / NN);
            const int node = (int)(idx - (long long)e * NN);
            const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
            const long long src = ni_gather_src(m, ni, e, idx);
            const bool own = ni_owner(ni);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const double bv = bp[c][src];
                double r = bv;
                if (applied) r = r - dss_value<N, double, DSS_CONT>(m, mx.Y64[c], ni, e, idx);
                mx.r64[c][idx] = r;
                mx.x32[c][idx] = 0.0f;
                if (own) {
                    part = fma(r, r, part);
                    if (want_b) partb = fma(bv, bv, partb);
                }
            }
        }
        double rr = 0.0, bbv = 0.0;
        grid_sum2_t<double>(part, partb, w.partials, slot, a.sync, a.timeout_ns, red, ok, rr, bbv);
        slot ^= 1;
        if (!ok) return false;
        if (threadIdx.x == 0) {
            const double rn = sqrt(rr);
            if (sweep == 0) sweep_state[0] = want_b ? sqrt(bbv) : rn;
            sweep_state[1] = rn;
            const double r0 = sweep_state[0];
            const bool c = rn < mx.outer_scale * (a.tol * r0 + a.tol);
            sweep_state[2] = (c || sweep >= mx.max_sweeps || inner_total >= a.maxit) ? (c ? 2.0 : 1.0) : 0.0;
        }
        __syncthreads();
        if (sweep_state[2] != 0.0) {
            conv = sweep_state[2] == 2.0;
            break;
        }
        // ---- FP32 inner solve A d = r (relative tolerance inner_tol)
        load_dmat_raw<N, float>(sm32, m);
        if (OP == OP_RES && mx.fdm) load_fdm_basis<N, float>(fdmS, fdmL, m);
        __syncthreads();
        const double* r64c[2] = {mx.r64[0], mx.r64[1]};
        auto rhs = [&](const NodeInfo&, int, long long flat, int c) -> float { return (float)r64c[c][flat]; };
        MinresOut ir{};
        const int budget = min(mx.inner_maxit, a.maxit - inner_total);
        // the inner solve reduces by inner_tol, or (last sweep) by no more
        // than the outer test still needs, with a margin for the FP32
        // estimate: a good initial guess then saves iterations, not sweeps
        double itol = mx.inner_tol;
        if (mx.adaptive) {
            const double need = mx.outer_scale * (a.tol * sweep_state[0] + a.tol) / sweep_state[1];
            itol = fmax(itol, fmin(0.3 * need, 0.5));
        }
        bool okc = false;
        bool done_fdm = false;
        if constexpr (OP == OP_RES) {
            if (mx.fdm) {
                okc = minres_core<N, float, OP, 2>(sm32, kmax, red, sc, m, mx.pot32, (float)a.alpha, eb, ee, w,
                                                   a.sync, a.timeout_ns, slot, rhs, mx.x32, budget, itol,
                                                   0.0, ir, (const float*)nullptr, fdmS, fdmL);
                done_fdm = true;
            }
        }
        if (done_fdm) {
        } else if constexpr (LEAN) {  // batched instances: no preconditioner or the element one
            okc = minres_core<N, float, OP, 0>(sm32, kmax, red, sc, m, mx.pot32, (float)a.alpha, eb, ee, w, a.sync,
                                               a.timeout_ns, slot, rhs, mx.x32, budget, itol, 0.0, ir,
                                               (const float*)nullptr);
        } else if (OP == OP_RES && mx.fused)
            okc = mx.pinv32
                      ? minres_core_fused<N, float, OP, true>(sm32, kmax, red, sc, m, mx.pot32, (float)a.alpha, eb,
                                                              ee, w, a.sync, a.timeout_ns, slot, rhs, mx.x32,
                                                              budget, itol, 0.0, ir, mx.pinv32)
                      : minres_core_fused<N, float, OP, false>(sm32, kmax, red, sc, m, mx.pot32, (float)a.alpha,
                                                               eb, ee, w, a.sync, a.timeout_ns, slot, rhs, mx.x32,
                                                               budget, itol, 0.0, ir, (const float*)nullptr);
        else
            okc = mx.pinv32
                      ? minres_core<N, float, OP, 1>(sm32, kmax, red, sc, m, mx.pot32, (float)a.alpha, eb, ee,
                                                        w, a.sync, a.timeout_ns, slot, rhs, mx.x32, budget,
                                                        itol, 0.0, ir, mx.pinv32)
                      : minres_core<N, float, OP, 0>(sm32, kmax, red, sc, m, mx.pot32, (float)a.alpha, eb, ee,
                                                         w, a.sync, a.timeout_ns, slot, rhs, mx.x32, budget,
                                                         itol, 0.0, ir, (const float*)nullptr);
        if (!okc) return false;
        inner_total += ir.it;
        ++sweep;
        // ---- x += d (FP64, owner copies; d is zero on the others)
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
#pragma unroll
            for (int c = 0; c < NC; ++c) xp[c][idx] += (double)mx.x32[c][idx];
        }
        if (!grid_barrier(a.sync, a.timeout_ns)) return false;
    }
    if (leader && threadIdx.x == 0) {
        a.out->success = conv ? 1 : 0;
        a.out->n_iter = inner_total;
        a.out->residual = sweep_state[1];
        a.out->status = 0;
        a.out->inner_iters = inner_total;
        a.out->sweeps = sweep;
    }
    __syncthreads();
    return true;
}

template <int N, int OP>
__global__ void __launch_bounds__(SOLVER_TPB, 1)
    k_minres_mixed(DevMesh m, SolveArgs a, KrylovWork<float> w, MixedArgs mx)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[34];
    __shared__ MinresScal<float> sc;
    __shared__ double sweep_state[3];  // r0, |r|, done
    __shared__ float fdmS[N * N], fdmL[N];  // element preconditioner basis
    int eb, ee;
    block_range(m.E, eb, ee);
    mixed_solve<N, OP>(m, a, w, mx, eb, ee, blockIdx.x == 0, smraw, red, sc, sweep_state, fdmS, fdmL);
}

// --------------------------------------------------------- persistent PCG
// include/pcg.hpp:59-97 with the identity preconditioner.  Vectors r, p in
// the continuous format; three grid barriers per iteration.
template <int N, typename T>
__global__ void __launch_bounds__(SOLVER_TPB, 1)
    k_pcg(DevMesh m, SolveArgs a, KrylovWork<T> w)
{
    constexpr int NN = N * N;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[34];
    __shared__ double ps[4];  // rho, rho_prev, bnorm, stop flag
    __shared__ T pc[2];       // beta, alpha of the current iteration
    T* sm = (T*)smraw;
    load_dmat_raw<N, T>(sm, m);
    __syncthreads();
    const Fac<T> fac = fac_of<T>(m);
    const T* b = (const T*)a.b[0];
    T* x = (T*)a.x[0];
    T* R = w.L[0];
    T* Pv = w.L[1];
    int eb, ee;
    block_range(m.E, eb, ee);
    const long long nb = (long long)eb * NN, ne = (long long)ee * NN;
    const int kmax = a.kmax;
    int slot = 0;
    bool ok = true;
    auto store_y = [&](T* Yb) {
        return [=](int, int, int, long long flat, const T* o) { Yb[flat] = o[0]; };
    };
    if (!a.x_is_zero) {
        for (int e0 = eb; e0 < ee; e0 += kmax)
            apply_range<N, T, OP_LAPLACE>(
                sm, kmax, fac, (const T*)nullptr, T(0), e0, min(kmax, ee - e0),
                [&](int e, int i, int j, long long flat, T* u) {
                    u[0] = x[ni_gather_src(m, node_info<N>(m, e, i, j), e, flat)];
                },
                store_y(w.Y[1]));
        if (!grid_barrier(a.sync, a.timeout_ns)) return;
    }
    T pb = T(0), pr = T(0);
    for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
        const int e = (int)(idx / NN);
        const int node = (int)(idx - (long long)e * NN);
        const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
        const T bv = b[ni_gather_src(m, ni, e, idx)];
        T r = bv;
        if (!a.x_is_zero) r = bv - dss_value<N, T, DSS_CONT>(m, w.Y[1], ni, e, idx);
        R[idx] = r;
        if (ni_owner(ni)) {
            pb = fma(bv, bv, pb);
            pr = fma(r, r, pr);
        }
    }
    double bb = 0.0, rho0 = 0.0;
    grid_sum2_t<T>(pb, pr, w.partials, slot, a.sync, a.timeout_ns, red, ok, bb, rho0);
    slot ^= 1;
    if (!ok) return;
    if (threadIdx.x == 0) {
        ps[0] = rho0;
        ps[1] = 0.0;
        ps[2] = sqrt(bb);
        ps[3] = 0.0;
        pc[0] = T(0);
    }
    __syncthreads();
    bool conv = false;
    int it = 0;
    double dummy = 0.0;
    for (it = 0; it < a.maxit; ++it) {
        const T beta = pc[0];
        for (int e0 = eb; e0 < ee; e0 += kmax)
            apply_range<N, T, OP_LAPLACE>(
                sm, kmax, fac, (const T*)nullptr, T(0), e0, min(kmax, ee - e0),
                [&](int, int, int, long long flat, T* u) {
                    const T pv = (it == 0) ? R[flat] : R[flat] + beta * Pv[flat];
                    Pv[flat] = pv;
                    u[0] = pv;
                },
                store_y(w.Y[0]));
        // the assembly below reads other blocks' element outputs
        if (!grid_barrier(a.sync, a.timeout_ns)) return;
        T pap = T(0);
#pragma unroll 4
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
            const int e = (int)(idx / NN);
            const int node = (int)(idx - (long long)e * NN);
            const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
            if (ni_owner(ni)) pap = fma(Pv[idx], dss_value<N, T, DSS_CONT>(m, w.Y[0], ni, e, idx), pap);
        }
        double pAp = 0.0;
        grid_sum2_t<T>(pap, T(0), w.partials, slot, a.sync, a.timeout_ns, red, ok, pAp, dummy);
        slot ^= 1;
        if (!ok) return;
        if (threadIdx.x == 0) pc[1] = (T)(ps[0] / pAp);
        __syncthreads();
        const T al = pc[1];
        T prr = T(0);
#pragma unroll 4
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
            const int e = (int)(idx / NN);
            const int node = (int)(idx - (long long)e * NN);
            const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
            const bool own = ni_owner(ni);
            const T ap = dss_value<N, T, DSS_CONT>(m, w.Y[0], ni, e, idx);
            if (own) x[idx] += al * Pv[idx];
            const T r = R[idx] - al * ap;
            R[idx] = r;
            if (own) prr = fma(r, r, prr);
        }
        if (threadIdx.x == 0) {
            ps[1] = ps[0];  // rho_prev = rho
            ps[3] = sqrt(ps[0]) < a.tol * ps[2] ? 1.0 : 0.0;  // pcg.hpp:84, rho of this iteration's start
        }
        __syncthreads();
        conv = ps[3] != 0.0;
        if (conv) break;
        double rho = 0.0;
        grid_sum2_t<T>(prr, T(0), w.partials, slot, a.sync, a.timeout_ns, red, ok, rho, dummy);
        slot ^= 1;
        if (!ok) return;
        if (threadIdx.x == 0) {
            pc[0] = (T)(rho / ps[1]);
            ps[0] = rho;
        }
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->success = conv ? 1 : 0;
        a.out->n_iter = it;
        a.out->residual = sqrt(ps[1]);  // rho of the last iteration's start (pcg.hpp:93)
        a.out->status = 0;
    }
}

// ------------------------------------------------------------- launchers

// dynamic shared memory of a solver kernel for a given staging capacity
template <int N>
size_t solver_smem(int op, bool mixed, int kmax)
{
    const bool two = (op == OP_RES);
    const size_t d = two ? range_smem_bytes<N, double, OP_RES>(kmax) : range_smem_bytes<N, double, OP_HELM>(kmax);
    const size_t f = two ? range_smem_bytes<N, float, OP_RES>(kmax) : range_smem_bytes<N, float, OP_HELM>(kmax);
    return mixed ? (d > f ? d : f) : d;
}

template <int N>
static const void* solver_fn(int op, bool mixed)
{
    if (mixed) return op == OP_RES ? (const void*)k_minres_mixed<N, OP_RES> : (const void*)k_minres_mixed<N, OP_HELM>;
    switch (op) {
        case OP_RES: return (const void*)k_minres<N, double, OP_RES>;
        case OP_HELM: return (const void*)k_minres<N, double, OP_HELM>;
        default: return (const void*)k_pcg<N, double>;
    }
}

// Plan a cooperative launch: one block per SM (fewer for small meshes) and
// the largest staging capacity kmax <= the block's element count that fits
// in smem_budget bytes.  Returns the grid, or 0 on failure.
template <int N>
int solver_plan(int op, bool mixed, int E, int sms, size_t smem_budget, int* kmax_out, size_t* smem_out)
{
    int grid = E < sms ? E : sms;
    if (grid < 1) grid = 1;
    int kmax = (E + grid - 1) / grid;
    while (kmax > 1 && solver_smem<N>(op, mixed, kmax) > smem_budget) kmax = (kmax + 1) / 2;
    const size_t smem = solver_smem<N>(op, mixed, kmax);
    const void* fn = solver_fn<N>(op, mixed);
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, SOLVER_TPB, smem) != cudaSuccess || per_sm < 1)
        return 0;
    *kmax_out = kmax;
    *smem_out = smem;
    return grid;
}

template <int N>
cudaError_t launch_solver(const DevMesh& m, const SolveArgs& a, const void* work, const MixedArgs* mx,
                          int grid, size_t smem, cudaStream_t st)
{
    DevMesh mm = m;
    SolveArgs aa = a;
    const bool mixed = mx != nullptr;
    const void* fn = solver_fn<N>(a.op, mixed);
    if (mixed) {
        KrylovWork<float> ww = *(const KrylovWork<float>*)work;
        MixedArgs xx = *mx;
        void* args[] = {&mm, &aa, &ww, &xx};
        return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(SOLVER_TPB), args, smem, st);
    }
    KrylovWork<double> ww = *(const KrylovWork<double>*)work;
    void* args[] = {&mm, &aa, &ww};
    return cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(SOLVER_TPB), args, smem, st);
}

}  // namespace semgb
