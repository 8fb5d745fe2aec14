// Persistent (cooperative) Krylov solvers: MINRES (FP64 or FP32), PCG, and
// FP64 iterative refinement around an FP32 inner MINRES.  One block per SM,
// SOLVER_TPB threads; each block owns a contiguous element range and stages
// up to kmax of its elements per pass in dynamic shared memory
// (apply_range).  Grid-wide phases are separated by bounded grid barriers.
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
template <int N, typename T, int OP, bool PRE, class Rhs>
__device__ __forceinline__ bool minres_core(T* sm, int kmax, double* red, const DevMesh& m,
                                            const T* pot, T alpha, int eb, int ee,
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
    double part = 0.0, partz = 0.0;
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
                    L[ir2][c * n + flat] = r;
                    W[iw1][c * n + flat] = T(0);
                    W[iw2][c * n + flat] = T(0);
                    const T z = PRE ? pv * r : r;
                    u[c] = z;
                    if (own) {
                        part = fma((double)r, (double)r, part);
                        if (PRE) partz = fma((double)r, (double)z, partz);
                    }
                }
            },
            store_y(w.Y[0]));
    const double bb = grid_sum(part, w.partials, slot, gs, tmo, red, ok);
    slot ^= 1;
    if (!ok) return false;
    double bz = bb;
    if (PRE) {
        bz = grid_sum(partz, w.partials, slot, gs, tmo, red, ok);
        slot ^= 1;
        if (!ok) return false;
    }

    const double eps_mach = (double)std::numeric_limits<T>::epsilon();
    const double bnorm = sqrt(bb);  // minres.hpp:28 (Euclidean, for the stopping test)
    const double beta1 = sqrt(bz);  // minres.hpp:31, sqrt(y.r1) with y = P^-1 r1
    double beta = beta1, beta_old = 0.0, phibar = beta1, cs = -1.0, sn = 0.0, dbar = 0.0, eps = 0.0;
    double pg = 0.0, peps = 0.0, pdelta = 0.0, pphi = 0.0, pinvb = 0.0;
    bool pending = false, conv = false;
    int it = 1;
    if (maxit >= 1) {
        for (;;) {
            // ---- Phase B_it
            const T inv_b = (T)(1.0 / beta);
            const T c1 = (T)(it >= 2 ? beta / beta_old : 0.0);
            const T* Ycur = w.Y[(it - 1) & 1];
            double s1 = 0.0;
#pragma unroll 4
            for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
                const int e = (int)(idx / NN);
                const int node = (int)(idx - (long long)e * NN);
                const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
                const bool own = ni_owner(ni);
                const T pv = PRE ? pinv[idx] : T(1);
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
                    const T vv = inv_b * (PRE ? pv * L[ir2][q] : L[ir2][q]);
                    if (own) s1 = fma((double)vv, (double)y3, s1);
                    L[iy][q] = y3;
                    if (pending) {
                        const T vprev = (T)pinvb * (PRE ? pv * r1v : r1v);
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
            const double alpha_i = grid_sum(s1, w.partials, slot, gs, tmo, red, ok);
            slot ^= 1;
            if (!ok) return false;
            // ---- Phase A_it+1
            const T c2 = (T)(alpha_i / beta);
            double ss = 0.0;
            T* Ynext = w.Y[it & 1];
            for (int e0 = eb; e0 < ee; e0 += kmax)
                apply_range<N, T, OP>(
                    sm, kmax, fac, pot, alpha, e0, min(kmax, ee - e0),
                    [&](int e, int i, int j, long long flat, T* u) {
                        const bool own = ni_owner(node_info<N>(m, e, i, j));
                        const T pv = PRE ? pinv[flat] : T(1);
#pragma unroll
                        for (int c = 0; c < NC; ++c) {
                            const long long q = c * n + flat;
                            const T y5 = L[iy][q] - c2 * L[ir2][q];
                            L[iy][q] = y5;
                            const T z = PRE ? pv * y5 : y5;  // y = precond(r2), minres.hpp:60
                            u[c] = z;
                            if (own) ss = fma((double)y5, (double)z, ss);
                        }
                    },
                    store_y(Ynext));
            const double bnew2 = grid_sum(ss, w.partials, slot, gs, tmo, red, ok);
            slot ^= 1;
            if (!ok) return false;
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
            conv = phibar < tol_rel * bnorm + tol_abs;  // minres.hpp:92
            if (conv || it == maxit) break;
            ++it;
        }
        // ---- Phase F: w/x update of the last iteration
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
            const int e = (int)(idx / NN);
            const int node = (int)(idx - (long long)e * NN);
            const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
            if (!ni_owner(ni)) continue;
            const T pv = PRE ? pinv[idx] : T(1);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                const long long q = c * n + idx;
                const T vprev = (T)pinvb * (PRE ? pv * L[ir1][q] : L[ir1][q]);
                const T wn = (T)pg * ((vprev - (T)peps * W[iw1][q]) - (T)pdelta * W[iw2][q]);
                xp[c][idx] += (T)pphi * wn;
            }
        }
    }
    res.it = it;
    res.phibar = phibar;
    res.conv = conv;
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
    if (!minres_core<N, T, OP, false>(sm, kmax, red, m, pot, alpha, eb, ee, w, a.sync, a.timeout_ns,
                                      slot, rhs, xp, a.maxit, a.tol, a.tol, r, (const T*)nullptr))
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
// with the true residual in place of the recursive estimate); else solve
// A d = r in FP32 to relative tolerance inner_tol and add d to x in FP64 on
// owner copies.
template <int N, int OP>
__global__ void __launch_bounds__(SOLVER_TPB, 1)
    k_minres_mixed(DevMesh m, SolveArgs a, KrylovWork<float> w, MixedArgs mx)
{
    constexpr int NN = N * N;
    constexpr int NC = op_nc<OP>();
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double red[34];
    double* sm64 = (double*)smraw;
    float* sm32 = (float*)smraw;
    const Fac<double> fac64 = fac_of<double>(m);
    const double* pot64 = (const double*)a.pot;
    const double* bp[2] = {(const double*)a.b[0], (const double*)a.b[1]};
    double* xp[2] = {(double*)a.x[0], (double*)a.x[1]};
    int eb, ee;
    block_range(m.E, eb, ee);
    const long long nb = (long long)eb * NN, ne = (long long)ee * NN;
    const int kmax = a.kmax;
    int slot = 0;
    bool ok = true;
    double r0 = 0.0, rn = 0.0;
    bool conv = false;
    int sweep = 0, inner_total = 0;
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
            if (!grid_barrier(a.sync, a.timeout_ns)) return;
        }
        double part = 0.0;
#pragma unroll 4
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
            const int e = (int)(idx / NN);
            const int node = (int)(idx - (long long)e * NN);
            const NodeInfo ni = node_info<N>(m, e, node % N, node / N);
            const long long src = ni_gather_src(m, ni, e, idx);
            const bool own = ni_owner(ni);
#pragma unroll
            for (int c = 0; c < NC; ++c) {
                double r = bp[c][src];
                if (applied) r = r - dss_value<N, double, DSS_CONT>(m, mx.Y64[c], ni, e, idx);
                mx.r64[c][idx] = r;
                mx.x32[c][idx] = 0.0f;
                if (own) part = fma(r, r, part);
            }
        }
        rn = sqrt(grid_sum(part, w.partials, slot, a.sync, a.timeout_ns, red, ok));
        slot ^= 1;
        if (!ok) return;
        if (sweep == 0) r0 = rn;
        conv = rn < a.tol * r0 + a.tol;
        if (conv || sweep >= mx.max_sweeps || inner_total >= a.maxit) break;
        // ---- FP32 inner solve A d = r (relative tolerance inner_tol)
        load_dmat_raw<N, float>(sm32, m);
        __syncthreads();
        const double* r64c[2] = {mx.r64[0], mx.r64[1]};
        auto rhs = [&](const NodeInfo&, int, long long flat, int c) -> float { return (float)r64c[c][flat]; };
        MinresOut ir{};
        const int budget = min(mx.inner_maxit, a.maxit - inner_total);
        const bool okc = mx.pinv32
                             ? minres_core<N, float, OP, true>(sm32, kmax, red, m, mx.pot32, (float)a.alpha, eb, ee,
                                                               w, a.sync, a.timeout_ns, slot, rhs, mx.x32, budget,
                                                               mx.inner_tol, 0.0, ir, mx.pinv32)
                             : minres_core<N, float, OP, false>(sm32, kmax, red, m, mx.pot32, (float)a.alpha, eb,
                                                                ee, w, a.sync, a.timeout_ns, slot, rhs, mx.x32,
                                                                budget, mx.inner_tol, 0.0, ir, (const float*)nullptr);
        if (!okc) return;
        inner_total += ir.it;
        ++sweep;
        // ---- x += d (FP64, owner copies; d is zero on the others)
        for (long long idx = nb + threadIdx.x; idx < ne; idx += blockDim.x) {
#pragma unroll
            for (int c = 0; c < NC; ++c) xp[c][idx] += (double)mx.x32[c][idx];
        }
        if (!grid_barrier(a.sync, a.timeout_ns)) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.out->success = conv ? 1 : 0;
        a.out->n_iter = inner_total;
        a.out->residual = rn;
        a.out->status = 0;
        a.out->inner_iters = inner_total;
        a.out->sweeps = sweep;
    }
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
        double pap = 0.0;
#pragma unroll 4
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
