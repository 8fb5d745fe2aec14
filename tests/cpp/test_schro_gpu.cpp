// The reference's test-suite (tests/*.cpp) re-run against the GPU library
// through the C++ layer include/schro_gpu/schro_gpu.hpp: same problems, same
// pass criteria.  Usage: test_schro_gpu <small_mesh folder>.  Exit status is
// the number of failed tests.
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "schro_gpu/schro_gpu.hpp"

using namespace schro_gpu;
using mat = matrix<double>;

static std::string g_mesh;

// host vector with the algebra the generic solvers need
struct hvec {
    std::vector<double> v;
    hvec() = default;
    explicit hvec(std::size_t n, double x = 0) : v(n, x) {}
    hvec& operator+=(const hvec& o) { for (std::size_t i = 0; i < v.size(); ++i) v[i] += o.v[i]; return *this; }
    hvec& operator-=(const hvec& o) { for (std::size_t i = 0; i < v.size(); ++i) v[i] -= o.v[i]; return *this; }
    friend hvec operator+(hvec a, const hvec& b) { return a += b; }
    friend hvec operator-(hvec a, const hvec& b) { return a -= b; }
    friend hvec operator*(double s, hvec a) { for (auto& x : a.v) x *= s; return a; }
};
static double hdot(const hvec& a, const hvec& b)
{
    double s = 0;
    for (std::size_t i = 0; i < a.v.size(); ++i) s += a.v[i] * b.v[i];
    return s;
}

// finite-difference -u'' - k u on n points (tests/pcg.cpp, tests/minres.cpp)
static hvec fd(const hvec& u, double h, double k)
{
    const std::size_t n = u.v.size();
    hvec r(n);
    for (std::size_t i = 0; i < n; ++i) {
        double s = 2 * u.v[i];
        if (i > 0) s -= u.v[i - 1];
        if (i + 1 < n) s -= u.v[i + 1];
        r.v[i] = s / (h * h) - k * u.v[i];
    }
    return r;
}

static bool test_pcg()
{
    const int n = 20;
    const double h = 2.0 / (n - 1), tol = 1e-5;
    hvec f(n), u(n);
    for (int i = 0; i < n; ++i) f.v[i] = std::pow(-1 + i * h, 2);
    auto L = [&](const hvec& x) { return fd(x, h, 0.0); };
    pcg<double>(u, L, f, hdot, IdentityPreconditioner{}, n, tol);
    hvec r = L(u) - f;
    return std::sqrt(hdot(r, r)) <= tol * std::sqrt(hdot(f, f));
}

static bool test_minres()
{
    const int n = 20;
    const double h = 2.0 / (n - 1), tol = 1e-5;
    hvec f(n), u(n);
    for (int i = 0; i < n; ++i) f.v[i] = std::pow(-1 + i * h, 2);
    auto L = [&](const hvec& x) { return fd(x, h, 2.0); };
    minres<double>(u, L, f, hdot, IdentityPreconditioner{}, n, tol);
    hvec r = L(u) - f;
    return std::sqrt(hdot(r, r)) <= tol * std::sqrt(hdot(f, f));
}

// tests/glaplace.cpp: weak Laplacian of a constant vanishes (p = 5, [-1,1]^2)
static bool test_glaplace()
{
    Mesh<double> m = Mesh<double>::from_arrays(5, {-1, -1, 1, -1, 1, 1, -1, 1}, {0, 1, 2, 3});
    dvec u(m.handle(), m.n_local());
    std::vector<double> ones(m.n_local(), 1.0), out(m.n_local());
    u.upload(ones.data());
    laplace(u).download(out.data());
    for (double v : out)
        if (std::abs(v) >= 1e-10) return false;
    return true;
}

// tests/solution_wrapper.cpp on the device vector: x += 2(3x - 0.5x) = 6
static bool test_dvec_algebra()
{
    Mesh<double> m = Mesh<double>::from_arrays(1, {-1, -1, 1, -1, 1, 1, -1, 1}, {0, 1, 2, 3});
    dvec x(m.handle(), 12);
    std::vector<double> ones(12, 1.0), out(12);
    x.upload(ones.data());
    dvec y = 0.5 * x;
    x += 2.0 * (3.0 * x - y);
    x.download(out.data());
    return out[0] == 6.0 && out[11] == 6.0 && x.size() == 12;
}

// mpi_tests/dot.cpp: dot(1, 1) = number of degrees of freedom
static bool test_dot()
{
    auto m = load_mesh<Mesh<double>>(6, g_mesh);
    dvec u(m.handle(), m.n_local());
    std::vector<double> ones(m.n_local(), 1.0);
    u.upload(ones.data());
    return dot(m, u, u) == (double)m.dof();
}

static std::vector<mat> field(const Mesh<double>& m, double (*f)(double, double))
{
    std::vector<double> X, Y;
    m.node_coords(X, Y);
    const int N = m.N;
    std::vector<mat> a(m.n_elements(), mat(N, N));
    for (int e = 0; e < m.n_elements(); ++e)
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                const std::size_t k = (std::size_t)e * N * N + i + (std::size_t)j * N;
                a[e](i, j) = f(X[k], Y[k]);
            }
    return a;
}

// tests/poisson.cpp
static bool test_poisson()
{
    auto mesh = load_mesh<Mesh<double>>(6, g_mesh);
    mesh.compute_metrics();
    auto F = field(mesh, [](double x, double y) { return x * x - y * y; });
    std::vector<mat> u(mesh.n_elements(), mat(mesh.N, mesh.N));
    auto r = poisson<double>(u, F, mesh, mesh.dof(), 1e-10);
    std::printf("poisson returned after %d iteration with residual %g\n", r.n_iter, r.residual);
    return r.success;
}

// tests/helmholtz.cpp
static bool test_helmholtz()
{
    auto mesh = load_mesh<Mesh<double>>(6, g_mesh);
    mesh.compute_metrics();
    auto F = field(mesh, [](double x, double y) { return x * x - y * y; });
    auto c = field(mesh, [](double, double) { return -100.0 - std::sqrt(2.0); });
    std::vector<mat> u(mesh.n_elements(), mat(mesh.N, mesh.N));
    auto r = helmholtz<double>(u, c, F, mesh, mesh.dof() * 10, 1e-10);
    std::printf("helmholtz returned after %d iteration with residual %g\n", r.n_iter, r.residual);
    return r.success;
}

// the generic minres template driving the GPU operator one call at a time
// agrees with the fused device solver
static bool test_generic_minres_on_device()
{
    auto mesh = load_mesh<Mesh<double>>(4, g_mesh);
    auto F = field(mesh, [](double x, double y) { return std::sin(x) * std::cos(2 * y); });
    std::vector<double> ff = flatten(F, (std::size_t)mesh.N * mesh.N);
    dvec f(mesh.handle(), mesh.n_local());
    f.upload(ff.data());
    dvec b = gproj(f, mesh);
    dvec x = 0.0 * b;
    auto A = [&](const dvec& v) { return laplace(v); };
    auto d = [&](const dvec& a, const dvec& c) { return dot(mesh, a, c); };
    auto r = minres<double>(x, A, b, d, IdentityPreconditioner{}, 10 * mesh.dof(), 1e-10);
    dvec y = 0.0 * b;
    sem_solver_results rr{};
    check(sem_pcg_laplace(mesh.handle(), y.data(), b.data(), 10 * mesh.dof(), 1e-10, 1, &rr), "pcg");
    dvec diff = x - y;
    const double rel = std::sqrt(dot(mesh, diff, diff) / dot(mesh, y, y));
    std::printf("generic minres: %d iterations, fused pcg: %d, rel diff %.2e\n", r.n_iter, rr.n_iter, rel);
    return r.success && rr.success && rel < 1e-7;
}

static double u0(double x, double y) { return std::sin(M_PI * x) * std::sin(M_PI * y); }
static double zero(double, double) { return 0.0; }

template <typename Driver>
static bool test_schrodinger(const char* name, Driver drv)
{
    auto mesh = load_mesh<Mesh<double>>(3, g_mesh);
    mesh.compute_metrics();
    auto V = field(mesh, zero), pr = field(mesh, u0), pi = field(mesh, zero);
    const double T = 0.01;
    solver_opts<double> opts;
    opts.dt = T / 10;
    opts.max_iter = 20 * mesh.dof();
    opts.tol = 1e-8;
    opts.verbose = false;
    int steps = 0;
    auto cb = [&](const std::vector<mat>&, const std::vector<mat>&) { ++steps; return false; };
    std::printf("solving Schrodinger equation with %s...\n", name);
    const bool ok = drv(pr, pi, V, mesh, T, opts, cb);
    if (!ok) std::printf("schrodinger_%s failed test\n", name);
    return ok && steps == 10;
}

int main(int argc, char** argv)
{
    g_mesh = argc > 1 ? argv[1] : "tests/golden/small_mesh";
    int failed = 0;
    auto run = [&](const char* n, bool (*t)()) {
        bool ok = false;
        try {
            ok = t();
        } catch (const std::exception& e) {
            std::printf("%s threw: %s\n", n, e.what());
        }
        std::printf("%-28s %s\n", n, ok ? "passed" : "FAILED");
        failed += ok ? 0 : 1;
    };
    run("test_pcg", test_pcg);
    run("test_minres", test_minres);
    run("test_glaplace", test_glaplace);
    run("test_dvec_algebra", test_dvec_algebra);
    run("test_dot", test_dot);
    run("test_poisson", test_poisson);
    run("test_helmholtz", test_helmholtz);
    run("test_generic_minres_on_device", test_generic_minres_on_device);
    run("test_schrodinger_bdf2", [] {
        return test_schrodinger("bdf2", [](auto&... a) { return schrodinger_bdf2<double>(a...); });
    });
    run("test_schrodinger_dirk4s3", [] {
        return test_schrodinger("dirk4s3", [](auto&... a) { return schrodinger_dirk4s3<double>(a...); });
    });
    run("test_schrodinger_dirk4s5", [] {
        return test_schrodinger("dirk4s5", [](auto&... a) { return schrodinger_dirk4s5<double>(a...); });
    });
    if (!failed) std::printf("all tests passed! :)\n");
    return failed;
}
