// C ABI over the reference's own OpenMP implementation (schro_omp), compiled
// from its unmodified headers against the shims in oracle/ref/shim/.
//
// TEST INFRASTRUCTURE ONLY: this library is the reference itself, used to pin
// the oracle restatement (oracle/sem_oracle.c), to generate the golden
// fixtures under tests/golden/ref/, and as the timed CPU baseline.  Nothing in
// the product package loads it.
//
// Fields cross this boundary as E blocks of N*N doubles, each block the
// column-major memory of one arma::Mat (value (i, j) of element e at
// e*N*N + j*N + i).
//
// Where the reference computes through a closure local to a driver (the
// Schroedinger Res and f operators, include/openmp_impl/schrodinger.hpp:
// 31-67, 147-207, 306-366, and the Helmholtz operator,
// include/openmp_impl/helmholtz.hpp:32-52), the closure's element formula is
// restated below over the reference's own unmask / glaplace / global_sum /
// mask, in the closure's order of operations; everything else calls the
// reference's functions and drivers directly.
#include "openmp_impl/poisson.hpp"
#include "openmp_impl/helmholtz.hpp"
#include "openmp_impl/schrodinger.hpp"
#include "load_mesh.hpp"

#include <omp.h>

#include <chrono>
#include <cstdio>
#include <cstring>

using schro_omp::Mesh;
typedef double real;
typedef std::vector<matrix<real>> field;

// LAPACK's dsteqr_/ssteqr_ (include/gauss_lobatto.hpp:22-25) come from
// lapack_fwd.cpp.
extern "C" int sem_ref_lapack_open(const char* path, char* err, int errlen);

namespace
{
thread_local char g_err[512];

void set_err(const char* what)
{
    std::snprintf(g_err, sizeof g_err, "%s", what);
}

struct RefMesh
{
    Mesh<real> mesh;
};

field to_field(const Mesh<real>& m, const double* a)
{
    const int N = m.N;
    const size_t E = m.elements.size();
    field f(E, matrix<real>(N, N));
    if (a)
        for (size_t e = 0; e < E; ++e) std::memcpy(f[e].memptr(), a + e * N * N, sizeof(double) * N * N);
    return f;
}

void from_field(const field& f, double* a)
{
    for (size_t e = 0; e < f.size(); ++e)
        std::memcpy(a + e * f[e].n_elem, f[e].memptr(), sizeof(double) * f[e].n_elem);
}

// L(u) of the Schroedinger closures: glaplace + (W (u % V) W) % J
// (include/openmp_impl/schrodinger.hpp:37-43)
matrix<real> schro_L(const Mesh<real>& mesh, const field& V, const matrix<real>& u, int i)
{
    const auto& w = mesh.quadrature.w;
    matrix<real> proj_Vu = (arma::diagmat(w) * (u % V[i]) * arma::diagmat(w)) % mesh.elements[i].J;
    matrix<real> nlap = glaplace(u, mesh.elements[i], mesh.D, mesh.quadrature);
    return nlap + proj_Vu;
}

// the Res closure (include/openmp_impl/schrodinger.hpp:45-67)
schro_omp::v_wrapper<real> schro_res(const Mesh<real>& mesh, const field& V, real alpha,
                                     const schro_omp::v_wrapper<real>& q)
{
    const auto& w = mesh.quadrature.w;
    const int n = mesh.elements.size();
    schro_omp::v_wrapper<real> y = q;
    schro_omp::unmask(y[0].values, mesh);
    schro_omp::unmask(y[1].values, mesh);
#pragma omp parallel for if (n > 63) schedule(static)
    for (int i = 0; i < n; ++i)
    {
        matrix<real> u = std::move(y[0].values[i]);
        matrix<real> v = std::move(y[1].values[i]);
        matrix<real> proj_u = (arma::diagmat(w) * u * arma::diagmat(w)) % mesh.elements[i].J;
        matrix<real> proj_v = (arma::diagmat(w) * v * arma::diagmat(w)) % mesh.elements[i].J;
        y[0].values[i] = proj_u + alpha * schro_L(mesh, V, v, i);
        y[1].values[i] = alpha * schro_L(mesh, V, u, i) - proj_v;
    }
    schro_omp::global_sum(y[0].values, mesh);
    schro_omp::global_sum(y[1].values, mesh);
    schro_omp::mask(y[0].values, mesh);
    schro_omp::mask(y[1].values, mesh);
    return y;
}

// the f closure (include/openmp_impl/schrodinger.hpp:163-183)
schro_omp::v_wrapper<real> schro_f(const Mesh<real>& mesh, const field& V, const schro_omp::v_wrapper<real>& q)
{
    const int n = mesh.elements.size();
    schro_omp::v_wrapper<real> y = q;
    schro_omp::unmask(y[0].values, mesh);
    schro_omp::unmask(y[1].values, mesh);
#pragma omp parallel for if (n > 63) schedule(static)
    for (int i = 0; i < n; ++i)
    {
        matrix<real> u = std::move(y[0].values[i]);
        matrix<real> v = std::move(y[1].values[i]);
        y[0].values[i] = -schro_L(mesh, V, v, i);
        y[1].values[i] = -schro_L(mesh, V, u, i);
    }
    schro_omp::global_sum(y[0].values, mesh);
    schro_omp::global_sum(y[1].values, mesh);
    schro_omp::mask(y[0].values, mesh);
    schro_omp::mask(y[1].values, mesh);
    return y;
}

schro_omp::v_wrapper<real> make_pair_field(const Mesh<real>& m, const double* a, const double* b)
{
    schro_omp::v_wrapper<real> p;
    p.values.resize(2);
    p[0] = schro_omp::solution_wrapper<real>(to_field(m, a));
    p[1] = schro_omp::solution_wrapper<real>(to_field(m, b));
    return p;
}

// Per-step callback of the drivers (include/openmp_impl/schrodinger.hpp:
// 116-118): records the wall time of each step and stops after n steps, so
// exactly n steps run whatever rounding does to the driver's t < T test, or
// earlier, once the steps after the first `untimed` have taken budget_s
// seconds (budget_s <= 0: no budget).
struct StepClock
{
    int n_steps;
    int untimed;
    double budget_s;
    int* done;
    double* times;
    double* spent;
    std::chrono::steady_clock::time_point* last;
    bool operator()(const field&, const field&)
    {
        auto now = std::chrono::steady_clock::now();
        const double dt = std::chrono::duration<double>(now - *last).count();
        if (times) times[*done] = dt;
        if (*done >= untimed) *spent += dt;
        *last = now;
        ++*done;
        return *done >= n_steps || (budget_s > 0 && *done > untimed && *spent >= budget_s);
    }
};

template <class F>
int guarded(F f)
{
    try
    {
        return f();
    }
    catch (const std::exception& e)
    {
        set_err(e.what());
        return -1;
    }
}
}  // namespace

extern "C" {

const char* ref_last_error(void) { return g_err; }

// Points the dsteqr_/ssteqr_ forwarders at a LAPACK shared library.
int ref_set_lapack(const char* path)
{
    return sem_ref_lapack_open(path, g_err, (int)sizeof g_err);
}

void ref_set_threads(int n)
{
    omp_set_dynamic(0);
    omp_set_num_threads(n);
}

int ref_get_threads(void) { return omp_get_max_threads(); }

// load_mesh + Mesh::compute_metrics (include/load_mesh.hpp:76-209,
// include/openmp_impl/Mesh.hpp:70-75)
void* ref_mesh_load(int p, const char* folder)
{
    try
    {
        auto* r = new RefMesh{load_mesh<Mesh<real>>(p, folder)};
        r->mesh.compute_metrics();
        return r;
    }
    catch (const std::exception& e)
    {
        set_err(e.what());
        return nullptr;
    }
}

void ref_mesh_free(void* h) { delete static_cast<RefMesh*>(h); }

void ref_mesh_info(void* h, int* N, int* n_el, int* n_nodes, int* n_edges, int* dof)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    *N = m.N;
    *n_el = (int)m.elements.size();
    *n_nodes = (int)m.nodes.size();
    *n_edges = (int)m.edges.size();
    *dof = m.dof();
}

// quadrature nodes and weights (include/gauss_lobatto.hpp:43-126) and the
// derivative matrix (include/derivative_matrix.hpp:12-38), column-major
void ref_quadrature(void* h, double* x, double* w, double* D)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    for (int i = 0; i < m.N; ++i)
    {
        x[i] = m.quadrature.x[i];
        w[i] = m.quadrature.w[i];
    }
    std::memcpy(D, m.D.memptr(), sizeof(double) * m.N * m.N);
}

// J, A, B, C per element (include/Quad.hpp:27-55)
void ref_metrics(void* h, double* J, double* A, double* B, double* C)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    const size_t NN = (size_t)m.N * m.N;
    for (size_t e = 0; e < m.elements.size(); ++e)
    {
        std::memcpy(J + e * NN, m.elements[e].J.memptr(), sizeof(double) * NN);
        std::memcpy(A + e * NN, m.elements[e].A.memptr(), sizeof(double) * NN);
        std::memcpy(B + e * NN, m.elements[e].B.memptr(), sizeof(double) * NN);
        std::memcpy(C + e * NN, m.elements[e].C.memptr(), sizeof(double) * NN);
    }
}

// physical coordinates of every element-local node, as the reference's tests
// compute them (Quad::from_local_coo, include/Quad.hpp:57-62)
void ref_node_coords(void* h, double* X, double* Y)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    const int N = m.N;
    for (size_t e = 0; e < m.elements.size(); ++e)
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i)
            {
                auto [x, y] = m.elements[e].from_local_coo(m.quadrature.x[i], m.quadrature.x[j]);
                X[e * N * N + j * N + i] = x;
                Y[e * N * N + j * N + i] = y;
            }
}

// edges in the mesh's order: elements[2], element_sides[2], startIter,
// deltaIter, edge_type (include/Edge.hpp), 7 ints per edge; corner nodes:
// corner_type and the (element, i, j) list (include/CornerNode.hpp)
void ref_edges(void* h, int* out)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    for (size_t k = 0; k < m.edges.size(); ++k)
    {
        const Edge& ed = m.edges[k];
        const bool interior = ed.edge_type != BOUNDARY;
        int* o = out + 7 * k;
        o[0] = ed.elements[0];
        o[1] = interior ? ed.elements[1] : -1;
        o[2] = ed.element_sides[0];
        o[3] = interior ? ed.element_sides[1] : 0;
        o[4] = interior ? ed.startIter : 0;
        o[5] = interior ? ed.deltaIter : 0;
        o[6] = interior ? 0 : 1;
    }
}

int ref_node_count_links(void* h)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    int n = 0;
    for (const auto& nd : m.nodes) n += (int)nd.connected_elements.size();
    return n;
}

// per node: type (0 interior, 1 boundary) and CSR of (element, i, j)
void ref_nodes(void* h, int* type, int* ptr, int* el, int* ii, int* jj)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    int k = 0;
    ptr[0] = 0;
    for (size_t n = 0; n < m.nodes.size(); ++n)
    {
        type[n] = m.nodes[n].corner_type == BOUNDARY ? 1 : 0;
        for (const auto& c : m.nodes[n].connected_elements)
        {
            el[k] = c.element_id;
            ii[k] = c.i;
            jj[k] = c.j;
            ++k;
        }
        ptr[n + 1] = k;
    }
}

// ---- gather-scatter (include/openmp_impl/unmask.hpp, global_sum.hpp, mask.hpp)
void ref_unmask(void* h, double* a)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    field f = to_field(m, a);
    schro_omp::unmask(f, m);
    from_field(f, a);
}

void ref_global_sum(void* h, double* a)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    field f = to_field(m, a);
    schro_omp::global_sum(f, m);
    from_field(f, a);
}

void ref_mask(void* h, double* a)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    field f = to_field(m, a);
    schro_omp::mask(f, m);
    from_field(f, a);
}

// include/openmp_impl/dot.hpp:11-61
double ref_dot(void* h, const double* a, const double* b)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    return schro_omp::dot(m, to_field(m, a), to_field(m, b));
}

// ---- element and assembled operators ----------------------------------------
// glaplace on every element, no assembly (include/glaplace.hpp:16-28)
void ref_glaplace(void* h, const double* u, double* out)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    field f = to_field(m, u);
    for (size_t e = 0; e < f.size(); ++e) f[e] = glaplace(f[e], m.elements[e], m.D, m.quadrature);
    from_field(f, out);
}

// include/openmp_impl/galerkin.hpp:42-57
void ref_gproj(void* h, const double* u, double* out)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    from_field(schro_omp::gproj<real>(to_field(m, u), m), out);
}

// Poisson's operator: galerkin_op over glaplace (include/openmp_impl/
// poisson.hpp:31-47, galerkin.hpp:24-35)
void ref_laplace_op(void* h, const double* u, double* out)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    auto op = [](field& v, const Mesh<real>& mesh) {
#pragma omp parallel for if (v.size() > 63) schedule(static)
        for (size_t i = 0; i < v.size(); ++i) v[i] = glaplace(v[i], mesh.elements[i], mesh.D, mesh.quadrature);
    };
    from_field(schro_omp::galerkin_op<real>(op, to_field(m, u), m), out);
}

// Helmholtz's operator (include/openmp_impl/helmholtz.hpp:32-52)
void ref_helmholtz_op(void* h, const double* c, const double* u, double* out)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    field cf = to_field(m, c);
    auto op = [&cf](field& v, const Mesh<real>& mesh) {
        const auto& w = mesh.quadrature.w;
#pragma omp parallel for if (v.size() > 63) schedule(static)
        for (size_t i = 0; i < v.size(); ++i)
        {
            matrix<real> cuv = (arma::diagmat(w) * (v[i] % cf[i]) * arma::diagmat(w)) % mesh.elements[i].J;
            v[i] = cuv + glaplace(v[i], mesh.elements[i], mesh.D, mesh.quadrature);
        }
    };
    from_field(schro_omp::galerkin_op<real>(op, to_field(m, u), m), out);
}

void ref_schro_res(void* h, const double* V, double alpha, const double* q0, const double* q1, double* y0,
                   double* y1)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    field Vf = to_field(m, V);
    auto y = schro_res(m, Vf, alpha, make_pair_field(m, q0, q1));
    from_field(y[0].values, y0);
    from_field(y[1].values, y1);
}

void ref_schro_f(void* h, const double* V, const double* q0, const double* q1, double* y0, double* y1)
{
    const auto& m = static_cast<RefMesh*>(h)->mesh;
    field Vf = to_field(m, V);
    auto y = schro_f(m, Vf, make_pair_field(m, q0, q1));
    from_field(y[0].values, y0);
    from_field(y[1].values, y1);
}

// ---- solvers and drivers -----------------------------------------------------
// include/openmp_impl/poisson.hpp:17-59 (u in/out); returns success, -1 on error
int ref_poisson(void* h, double* u, const double* f, int maxit, double tol, int* n_iter, double* residual)
{
    return guarded([&] {
        const auto& m = static_cast<RefMesh*>(h)->mesh;
        field uf = to_field(m, u);
        auto r = schro_omp::poisson<real>(uf, to_field(m, f), m, maxit, tol);
        from_field(uf, u);
        *n_iter = r.n_iter;
        *residual = r.residual;
        return r.success ? 1 : 0;
    });
}

// include/openmp_impl/helmholtz.hpp:18-64
int ref_helmholtz(void* h, double* u, const double* c, const double* f, int maxit, double tol, int* n_iter,
                  double* residual)
{
    return guarded([&] {
        const auto& m = static_cast<RefMesh*>(h)->mesh;
        field uf = to_field(m, u);
        auto r = schro_omp::helmholtz<real>(uf, to_field(m, c), to_field(m, f), m, maxit, tol);
        from_field(uf, u);
        *n_iter = r.n_iter;
        *residual = r.residual;
        return r.success ? 1 : 0;
    });
}

// The reference's PCG (include/pcg.hpp:59-97) on Poisson's operator and its
// MINRES on Helmholtz's, with the drivers' dot product, for an arbitrary
// right-hand side b (the drivers build b = gproj(f) themselves,
// include/openmp_impl/poisson.hpp:20, helmholtz.hpp:21).  x in/out.
int ref_pcg_laplace(void* h, double* x, const double* b, int maxit, double tol, int* n_iter, double* residual)
{
    return guarded([&] {
        const auto& m = static_cast<RefMesh*>(h)->mesh;
        schro_omp::solution_wrapper<real> xs(to_field(m, x)), bs(to_field(m, b));
        auto op = [](field& v, const Mesh<real>& mesh) {
#pragma omp parallel for if (v.size() > 63) schedule(static)
            for (size_t i = 0; i < v.size(); ++i) v[i] = glaplace(v[i], mesh.elements[i], mesh.D, mesh.quadrature);
        };
        auto L = [&](const schro_omp::solution_wrapper<real>& v) {
            return schro_omp::solution_wrapper<real>(schro_omp::galerkin_op<real>(op, v.values, m));
        };
        auto dotprod = [&](const schro_omp::solution_wrapper<real>& a, const schro_omp::solution_wrapper<real>& c) {
            return schro_omp::dot<real>(m, a.values, c.values);
        };
        auto r = pcg<real>(xs, L, bs, dotprod, IdentityPreconditioner{}, maxit, tol);
        from_field(xs.values, x);
        *n_iter = r.n_iter;
        *residual = r.residual;
        return r.success ? 1 : 0;
    });
}

int ref_minres_helmholtz(void* h, const double* c, double* x, const double* b, int maxit, double tol, int* n_iter,
                         double* residual)
{
    return guarded([&] {
        const auto& m = static_cast<RefMesh*>(h)->mesh;
        field cf = to_field(m, c);
        schro_omp::solution_wrapper<real> xs(to_field(m, x)), bs(to_field(m, b));
        auto op = [&cf](field& v, const Mesh<real>& mesh) {
            const auto& w = mesh.quadrature.w;
#pragma omp parallel for if (v.size() > 63) schedule(static)
            for (size_t i = 0; i < v.size(); ++i)
            {
                matrix<real> cuv = (arma::diagmat(w) * (v[i] % cf[i]) * arma::diagmat(w)) % mesh.elements[i].J;
                v[i] = cuv + glaplace(v[i], mesh.elements[i], mesh.D, mesh.quadrature);
            }
        };
        auto A = [&](const schro_omp::solution_wrapper<real>& v) {
            return schro_omp::solution_wrapper<real>(schro_omp::galerkin_op<real>(op, v.values, m));
        };
        auto dotprod = [&](const schro_omp::solution_wrapper<real>& a, const schro_omp::solution_wrapper<real>& d) {
            return schro_omp::dot<real>(m, a.values, d.values);
        };
        auto r = minres<real>(xs, A, bs, dotprod, IdentityPreconditioner{}, maxit, tol);
        from_field(xs.values, x);
        *n_iter = r.n_iter;
        *residual = r.residual;
        return r.success ? 1 : 0;
    });
}

// The reference's MINRES (include/minres.hpp:19-107) on the Res operator
// with the drivers' dot product (include/openmp_impl/schrodinger.hpp:
// 368-371): x in/out
int ref_minres_res(void* h, const double* V, double alpha, const double* b0, const double* b1, double* x0,
                   double* x1, int maxit, double tol, int* n_iter, double* residual)
{
    return guarded([&] {
        const auto& m = static_cast<RefMesh*>(h)->mesh;
        field Vf = to_field(m, V);
        auto x = make_pair_field(m, x0, x1);
        auto b = make_pair_field(m, b0, b1);
        auto A = [&](const schro_omp::v_wrapper<real>& q) { return schro_res(m, Vf, alpha, q); };
        auto dotprod = [&](const schro_omp::v_wrapper<real>& a, const schro_omp::v_wrapper<real>& c) -> real {
            return schro_omp::dot<real>(m, a[0].values, c[0].values) + schro_omp::dot<real>(m, a[1].values, c[1].values);
        };
        auto r = minres<real>(x, A, b, dotprod, IdentityPreconditioner{}, maxit, tol);
        from_field(x[0].values, x0);
        from_field(x[1].values, x1);
        *n_iter = r.n_iter;
        *residual = r.residual;
        return r.success ? 1 : 0;
    });
}

// The drivers schrodinger_bdf2 (method 0), schrodinger_dirk4s3 (1) and
// schrodinger_dirk4s5 (2) (include/openmp_impl/schrodinger.hpp:22-128,
// 138-285, 294-423), run for n_steps steps of size dt through the driver's
// callback, or fewer when the steps after the first `untimed` reach budget_s
// seconds.  step_times (n_steps entries, may be null) receives the wall time
// of each step.  psi in/out.  Returns the driver's success flag.
int ref_schrodinger(void* h, int method, double* re, double* im, const double* V, double dt, int maxit,
                    double tol, int n_steps, int untimed, double budget_s, double* step_times, int* steps_done)
{
    return guarded([&] {
        const auto& m = static_cast<RefMesh*>(h)->mesh;
        field pr = to_field(m, re), pi = to_field(m, im), Vf = to_field(m, V);
        solver_opts<real> opts;
        opts.max_iter = maxit;
        opts.tol = tol;
        opts.dt = dt;
        opts.verbose = false;
        int done = 0;
        double spent = 0.0;
        auto last = std::chrono::steady_clock::now();
        StepClock cb{n_steps, untimed, budget_s, &done, step_times, &spent, &last};
        // T past the last step: the callback ends the run after n_steps
        const real T = dt * (n_steps + 1);
        bool ok;
        if (method == 0)
            ok = schro_omp::schrodinger_bdf2<real>(pr, pi, Vf, m, T, opts, cb);
        else if (method == 1)
            ok = schro_omp::schrodinger_dirk4s3<real>(pr, pi, Vf, m, T, opts, cb);
        else if (method == 2)
            ok = schro_omp::schrodinger_dirk4s5<real>(pr, pi, Vf, m, T, opts, cb);
        else
            throw std::invalid_argument("method must be 0 (bdf2), 1 (dirk4s3) or 2 (dirk4s5)");
        from_field(pr, re);
        from_field(pi, im);
        *steps_done = done;
        return ok ? 1 : 0;
    });
}

}  // extern "C"
