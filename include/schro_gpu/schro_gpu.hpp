// schro_gpu.hpp -- C++20 host layer over the C ABI of sem_gb300.h.
//
// Keeps the reference's template API (arotem3/SchrodingerSEM,
// include/solver_base.hpp, ode_base.hpp, Op.hpp, minres.hpp, pcg.hpp,
// load_mesh.hpp and openmp_impl/{poisson,helmholtz,schrodinger,dot,
// galerkin,unmask,global_sum,mask}.hpp) so code written against schro_omp
// compiles against schro_gpu by swapping the namespace:
//
//   schro_omp::Mesh<double> m = load_mesh<schro_omp::Mesh<double>>(p, dir);
//   -> auto m = schro_gpu::load_mesh<schro_gpu::Mesh<double>>(p, dir);
//
// Fields stay std::vector<matrix> (one column-major N x N block per element,
// any matrix type with memptr() and n_elem, e.g. arma::Mat or
// schro_gpu::matrix).  Every operator runs in the library's CUDA kernels;
// the generic minres/pcg templates below also accept schro_gpu::dvec, a
// device vector with the reference's expression algebra, so the same
// algorithm can drive the GPU operators one call at a time.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <concepts>
#include <cstring>
#include <functional>
#include <limits>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../sem_gb300.h"

namespace schro_gpu {

// ------------------------------------------------------------ basic types
// solver_results / IdentityPreconditioner (include/solver_base.hpp:6-22)
template <typename real>
struct solver_results {
    bool success;
    int n_iter;
    real residual;
};

class IdentityPreconditioner {
public:
    template <typename vec>
    vec operator()(const vec& x) { return x; }
};

// solver_opts / NullCallback (include/ode_base.hpp:6-23)
template <std::floating_point real>
struct solver_opts {
    int max_iter;
    real tol;
    real dt;
    bool verbose;
};

class NullCallback {
public:
    template <typename... Args>
    constexpr bool operator()(const Args&...) { return false; }
};

// element-wise operations of the expression algebra (include/Op.hpp:9-37)
template <typename V>
struct Plus { static V apply(const V& x, const V& y) { return x + y; } };
template <typename V>
struct Minus { static V apply(const V& x, const V& y) { return x - y; } };
template <typename S, typename V>
struct Scale { static V apply(const S& s, const V& x) { return s * x; } };

// minimal column-major dense matrix (stand-in for arma::Mat in user code)
template <typename T>
class matrix {
public:
    using elem_type = T;
    matrix() = default;
    matrix(std::size_t r, std::size_t c, T v = T(0)) : n_rows(r), n_cols(c), n_elem(r * c), d(r * c, v) {}
    T& at(std::size_t i, std::size_t j) { return d[i + j * n_rows]; }
    const T& at(std::size_t i, std::size_t j) const { return d[i + j * n_rows]; }
    T& operator()(std::size_t i, std::size_t j) { return at(i, j); }
    const T& operator()(std::size_t i, std::size_t j) const { return at(i, j); }
    T* memptr() { return d.data(); }
    const T* memptr() const { return d.data(); }
    std::size_t n_rows = 0, n_cols = 0, n_elem = 0;

private:
    std::vector<T> d;
};

// ----------------------------------------------------------------- errors
inline void check(int status, const char* where)
{
    if (status != SEM_OK)
        throw std::runtime_error(std::string(where) + ": " + sem_status_string(status) + " " + sem_last_error());
}

// ------------------------------------------------------------------- mesh
// schro_omp::Mesh (include/openmp_impl/Mesh.hpp:16-88) backed by a sem_ctx.
template <std::floating_point real>
class Mesh {
    static_assert(std::is_same_v<real, double>, "the GB300 library computes in double (mixed mode inside)");

public:
    typedef real real_t;

    Mesh() = default;
    Mesh(const Mesh&) = delete;
    Mesh& operator=(const Mesh&) = delete;
    Mesh(Mesh&& o) noexcept : ctx(o.ctx), info(o.info), x(std::move(o.x)), w(std::move(o.w)) { o.ctx = nullptr; }
    Mesh& operator=(Mesh&& o) noexcept
    {
        std::swap(ctx, o.ctx);
        info = o.info;
        x = std::move(o.x);
        w = std::move(o.w);
        return *this;
    }
    ~Mesh() { sem_ctx_destroy(ctx); }

    static Mesh from_arrays(int p, const std::vector<double>& coords, const std::vector<int>& elements,
                            unsigned flags = 0)
    {
        Mesh m;
        check(sem_ctx_create(&m.ctx, p, (int)(coords.size() / 2), coords.data(), (int)(elements.size() / 4),
                             elements.data(), flags),
              "sem_ctx_create");
        m.init();
        return m;
    }
    static Mesh from_folder(int p, const std::string& folder, unsigned flags = 0)
    {
        Mesh m;
        check(sem_ctx_load(&m.ctx, p, folder.c_str(), flags), "sem_ctx_load");
        m.init();
        return m;
    }

    // metrics are computed with the mesh (kept for source compatibility)
    void compute_metrics() {}
    int dof() const { return (int)info.dof; }
    int n_elements() const { return info.n_elements; }
    std::size_t n_local() const { return (std::size_t)info.n_local; }
    sem_ctx* handle() const { return ctx; }
    // Quad::from_local_coo at every node: x, y as flat E*N*N arrays
    void node_coords(std::vector<double>& X, std::vector<double>& Y) const
    {
        X.resize(n_local());
        Y.resize(n_local());
        check(sem_ctx_get_node_coords(ctx, X.data(), Y.data()), "sem_ctx_get_node_coords");
    }

    int N = 0;
    struct { std::vector<real> x, w; } quadrature;

private:
    void init()
    {
        check(sem_ctx_get_info(ctx, &info), "sem_ctx_get_info");
        N = info.N;
        x.resize(N);
        w.resize(N);
        check(sem_ctx_get_quadrature(ctx, x.data(), w.data(), nullptr), "sem_ctx_get_quadrature");
        quadrature.x = x;
        quadrature.w = w;
    }
    sem_ctx* ctx = nullptr;
    sem_mesh_info info{};
    std::vector<real> x, w;
};

// load_mesh<MeshT>(p, folder) (include/load_mesh.hpp:76-77)
template <typename MeshT>
MeshT load_mesh(int p, const std::string& folder)
{
    return MeshT::from_folder(p, folder);
}

// ------------------------------------------------------ host <-> flat fields
template <typename M>
std::vector<double> flatten(const std::vector<M>& a, std::size_t per)
{
    std::vector<double> f(a.size() * per);
    for (std::size_t e = 0; e < a.size(); ++e) {
        if ((std::size_t)a[e].n_elem != per) throw std::invalid_argument("field block has the wrong size");
        std::memcpy(f.data() + e * per, a[e].memptr(), per * sizeof(double));
    }
    return f;
}

template <typename M>
void unflatten(const double* f, std::vector<M>& a, std::size_t per)
{
    for (std::size_t e = 0; e < a.size(); ++e) std::memcpy(a[e].memptr(), f + e * per, per * sizeof(double));
}

// ------------------------------------------------------------ device vector
// A field on the device with the reference's vector algebra
// (solution_wrapper.hpp:20-201 + Op.hpp): copies, +, -, scalar *, +=, -=.
// Expressions are evaluated eagerly through sem_vec_axpby.
class dvec {
public:
    dvec() = default;
    dvec(sem_ctx* c, std::size_t n) : ctx(c), n(n) { alloc(); }
    dvec(const dvec& o) : ctx(o.ctx), n(o.n)
    {
        alloc();
        if (n) check_cuda(cudaMemcpy(p, o.p, bytes(), cudaMemcpyDeviceToDevice));
    }
    dvec(dvec&& o) noexcept : ctx(o.ctx), n(o.n), p(o.p) { o.p = nullptr; o.n = 0; }
    dvec& operator=(dvec o) noexcept
    {
        std::swap(ctx, o.ctx);
        std::swap(n, o.n);
        std::swap(p, o.p);
        return *this;
    }
    ~dvec() { if (p) cudaFree(p); }

    void upload(const double* h) { check_cuda(cudaMemcpy(p, h, bytes(), cudaMemcpyHostToDevice)); }
    void download(double* h) const { check_cuda(cudaMemcpy(h, p, bytes(), cudaMemcpyDeviceToHost)); }
    double* data() { return p; }
    const double* data() const { return p; }
    std::size_t size() const { return n; }
    sem_ctx* context() const { return ctx; }

    dvec& operator+=(const dvec& o) { return axpby(1.0, *this, 1.0, &o, *this); }
    dvec& operator-=(const dvec& o) { return axpby(1.0, *this, -1.0, &o, *this); }
    friend dvec operator+(const dvec& a, const dvec& b) { dvec r(a.ctx, a.n); axpby(1.0, a, 1.0, &b, r); return r; }
    friend dvec operator-(const dvec& a, const dvec& b) { dvec r(a.ctx, a.n); axpby(1.0, a, -1.0, &b, r); return r; }
    friend dvec operator*(double s, const dvec& a) { dvec r(a.ctx, a.n); axpby(s, a, 0.0, nullptr, r); return r; }
    friend dvec operator*(const dvec& a, double s) { return s * a; }

private:
    static dvec& axpby(double a, const dvec& x, double b, const dvec* y, dvec& out)
    {
        check(sem_vec_axpby(x.ctx, (long long)x.n, a, x.p, b, y ? y->p : nullptr, out.p), "sem_vec_axpby");
        return out;
    }
    static void check_cuda(cudaError_t e)
    {
        if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
    }
    void alloc()
    {
        if (n) check_cuda(cudaMalloc((void**)&p, bytes()));
    }
    std::size_t bytes() const { return n * sizeof(double); }
    sem_ctx* ctx = nullptr;
    std::size_t n = 0;
    double* p = nullptr;
};

// ------------------------------------------- generic Krylov solvers (host)
// MINRES of Paige & Saunders (SIAM J. Numer. Anal. 12, 1975) over any vector
// type with +, -, scalar * and +=: the same steps and stopping rule as the
// reference (include/minres.hpp:19-107), with the preconditioned recurrence
// beta = sqrt(r . M^-1 r).  Each A(v) / dot call is one GPU operation for
// dvec, so this is the "one call at a time" path; the fused solvers below
// (sem_minres_* and the drivers) run the whole iteration on the device.
template <std::floating_point real, typename vec, std::invocable<vec> LinOp, std::invocable<vec, vec> Dot,
          std::invocable<vec> Precond>
solver_results<real> minres(vec& x, LinOp A, const vec& b, Dot dot, Precond precond, int maxit, real tol)
{
    vec r_prev = b - A(x);
    vec z = precond(r_prev);
    vec r_cur = r_prev;
    const real r0 = std::sqrt(dot(r_prev, r_prev));
    const real beta1 = std::sqrt(dot(z, r_prev));
    real beta = beta1, beta_prev = 0, dbar = 0, eps = 0, phibar = beta1, c = -1, s = 0;
    vec d = real(0) * x;
    vec d_prev = d, d_prev2 = d;
    int it = 1;
    bool ok = false;
    for (; it <= maxit; ++it) {
        vec v = (real(1) / beta) * z;
        vec y = A(v);
        if (it >= 2) y -= (beta / beta_prev) * r_prev;
        const real a = dot(v, y);
        y -= (a / beta) * r_cur;
        r_prev = std::move(r_cur);
        r_cur = y;
        z = precond(r_cur);
        beta_prev = beta;
        beta = std::sqrt(dot(r_cur, z));
        const real eps_prev = eps;
        const real delta = c * dbar + s * a;
        const real gbar = s * dbar - c * a;
        eps = s * beta;
        dbar = -c * beta;
        const real gamma = std::max(std::sqrt(gbar * gbar + beta * beta), std::numeric_limits<real>::epsilon());
        c = gbar / gamma;
        s = beta / gamma;
        const real phi = c * phibar;
        phibar *= s;
        d_prev2 = std::move(d_prev);
        d_prev = std::move(d);
        d = (real(1) / gamma) * ((v - eps_prev * d_prev2) - delta * d_prev);
        x += phi * d;
        if (phibar < tol * r0 + tol) {
            ok = true;
            break;
        }
    }
    return {ok, it, phibar};
}

// Conjugate gradients (Saad, Iterative methods, 2003): the reference's
// pcg.hpp:59-97 steps and stopping rule (sqrt(rho) < tol |b| with rho taken
// at the start of the iteration).
template <std::floating_point real, typename vec, std::invocable<vec> LinOp, std::invocable<vec, vec> Dot,
          std::invocable<vec> Precond>
solver_results<real> pcg(vec& x, LinOp A, const vec& b, Dot dot, Precond precond, int max_iter, real tol)
{
    vec r = b - A(x);
    const real bn = std::sqrt(dot(b, b));
    vec p = r;
    real rho = 0, rho_prev = 0;
    int it = 0;
    bool ok = false;
    for (; it < max_iter; ++it) {
        vec z = precond(r);
        rho = dot(r, z);
        if (it == 0) p = z;
        else p = z + (rho / rho_prev) * p;
        vec Ap = A(p);
        const real al = rho / dot(p, Ap);
        x += al * p;
        r -= al * Ap;
        rho_prev = rho;
        if (std::sqrt(rho) < tol * bn) {
            ok = true;
            break;
        }
    }
    return {ok, it, std::sqrt(rho)};
}

// ------------------------------------------- gather-scatter and operators
// dot (openmp_impl/dot.hpp:11-61), unmask/global_sum/mask (unmask.hpp,
// global_sum.hpp, mask.hpp), gproj and the Galerkin operators on dvec.
inline double dot(const Mesh<double>&, const dvec& a, const dvec& b)
{
    double r = 0;
    check(sem_dot(a.context(), a.data(), b.data(), &r), "sem_dot");
    return r;
}
inline void unmask(dvec& a, const Mesh<double>&) { check(sem_unmask(a.context(), a.data()), "sem_unmask"); }
inline void global_sum(dvec& a, const Mesh<double>&) { check(sem_global_sum(a.context(), a.data()), "sem_global_sum"); }
inline void mask(dvec& a, const Mesh<double>&) { check(sem_mask(a.context(), a.data()), "sem_mask"); }
inline dvec gproj(const dvec& u, const Mesh<double>&)
{
    dvec r(u.context(), u.size());
    check(sem_gproj(u.context(), u.data(), r.data()), "sem_gproj");
    return r;
}
inline dvec laplace(const dvec& u)
{
    dvec r(u.context(), u.size());
    check(sem_apply_laplace(u.context(), u.data(), r.data()), "sem_apply_laplace");
    return r;
}

// ----------------------------------------------------------------- drivers
// schro_omp::poisson (openmp_impl/poisson.hpp:17-59)
template <std::floating_point real, typename M>
solver_results<real> poisson(std::vector<M>& u, const std::vector<M>& f, const Mesh<real>& mesh, int max_iter,
                             real tol)
{
    const std::size_t per = (std::size_t)mesh.N * mesh.N;
    std::vector<double> uf = flatten(u, per), ff = flatten(f, per);
    sem_solver_results r{};
    check(sem_poisson(mesh.handle(), uf.data(), ff.data(), max_iter, tol, &r), "sem_poisson");
    unflatten(uf.data(), u, per);
    return {r.success != 0, r.n_iter, (real)r.residual};
}

// schro_omp::helmholtz (openmp_impl/helmholtz.hpp:18-64)
template <std::floating_point real, typename M>
solver_results<real> helmholtz(std::vector<M>& u, const std::vector<M>& c, const std::vector<M>& f,
                               const Mesh<real>& mesh, int max_iter, real tol)
{
    const std::size_t per = (std::size_t)mesh.N * mesh.N;
    std::vector<double> uf = flatten(u, per), cf = flatten(c, per), ff = flatten(f, per);
    sem_solver_results r{};
    check(sem_helmholtz(mesh.handle(), uf.data(), cf.data(), ff.data(), max_iter, tol, &r), "sem_helmholtz");
    unflatten(uf.data(), u, per);
    return {r.success != 0, r.n_iter, (real)r.residual};
}

namespace detail {
template <typename M, typename Callback>
struct StepHook {
    Callback* cb;
    std::vector<M>* re;
    std::vector<M>* im;
    std::size_t per;
};

template <typename M, typename Callback>
int step_trampoline(void* user, int, const double* pr, const double* pi)
{
    auto* h = static_cast<StepHook<M, Callback>*>(user);
    unflatten(pr, *h->re, h->per);
    unflatten(pi, *h->im, h->per);
    return (*h->cb)(*h->re, *h->im) ? 1 : 0;
}

using driver_fn = int (*)(sem_ctx*, double*, double*, const double*, double, const sem_solver_opts*,
                          sem_step_callback, void*, int*);

template <typename real, typename M, typename Callback>
bool run_driver(driver_fn fn, std::vector<M>& psi_re, std::vector<M>& psi_im, const std::vector<M>& V,
                const Mesh<real>& mesh, real T, const solver_opts<real>& opts, Callback callback)
{
    const std::size_t per = (std::size_t)mesh.N * mesh.N;
    std::vector<double> pr = flatten(psi_re, per), pi = flatten(psi_im, per), vf = flatten(V, per);
    sem_solver_opts o{opts.max_iter, (double)opts.tol, (double)opts.dt, opts.verbose ? 1 : 0};
    StepHook<M, Callback> hook{&callback, &psi_re, &psi_im, per};
    const bool null_cb = std::is_same_v<Callback, NullCallback>;
    int ok = 0;
    check(fn(mesh.handle(), pr.data(), pi.data(), vf.data(), (double)T, &o,
             null_cb ? nullptr : &step_trampoline<M, Callback>, &hook, &ok),
          "sem_schrodinger");
    unflatten(pr.data(), psi_re, per);
    unflatten(pi.data(), psi_im, per);
    return ok != 0;
}
}  // namespace detail

// schro_omp::schrodinger_bdf2 / _dirk4s5 / _dirk4s3
// (openmp_impl/schrodinger.hpp:22-128, 138-285, 294-423)
template <std::floating_point real, typename M, typename Callback = NullCallback>
bool schrodinger_bdf2(std::vector<M>& psi_real, std::vector<M>& psi_imag, const std::vector<M>& potential,
                      const Mesh<real>& mesh, real T, const solver_opts<real>& opts, Callback callback = {})
{
    return detail::run_driver(&sem_schrodinger_bdf2, psi_real, psi_imag, potential, mesh, T, opts, callback);
}
template <std::floating_point real, typename M, typename Callback = NullCallback>
bool schrodinger_dirk4s5(std::vector<M>& psi_real, std::vector<M>& psi_imag, const std::vector<M>& potential,
                         const Mesh<real>& mesh, real T, const solver_opts<real>& opts, Callback callback = {})
{
    return detail::run_driver(&sem_schrodinger_dirk4s5, psi_real, psi_imag, potential, mesh, T, opts, callback);
}
template <std::floating_point real, typename M, typename Callback = NullCallback>
bool schrodinger_dirk4s3(std::vector<M>& psi_real, std::vector<M>& psi_imag, const std::vector<M>& potential,
                         const Mesh<real>& mesh, real T, const solver_opts<real>& opts, Callback callback = {})
{
    return detail::run_driver(&sem_schrodinger_dirk4s3, psi_real, psi_imag, potential, mesh, T, opts, callback);
}

}  // namespace schro_gpu
