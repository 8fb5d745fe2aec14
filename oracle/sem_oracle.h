/*
 * sem_oracle.h -- CPU restatement of arotem3/SchrodingerSEM's OpenMP path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the CUDA library is
 * compared against: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The product never links or calls it.
 *
 * Parity pinning: the reference needs Armadillo, Boost.Math, Boost.MPI and
 * LAPACK, none of which exist on this machine, so it cannot be compiled
 * here.  This restatement is pinned instead against every known-answer test
 * the reference's own test-suite holds for the path (tests/gauss_lobatto.cpp,
 * tests/derivative_matrix.cpp, tests/glaplace.cpp, tests/pcg.cpp,
 * tests/minres.cpp, mpi_tests/dot.cpp, and the convergence tests of
 * tests/poisson.cpp, tests/helmholtz.cpp, tests/schrodinger.cpp on the
 * reference's sample mesh).
 *
 * Data layout (same as the reference's std::vector<arma::Mat>): a field is E
 * column-major N x N blocks, value (i,j) of element e at a[e*N*N + j*N + i],
 * i the xi index and j the eta index.
 */
#ifndef SEM_ORACLE_H
#define SEM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* include/MeshBase.hpp:5-8 */
enum { OR_INTERIOR = 0, OR_BOUNDARY = 1 };

typedef struct or_mesh {
    int p, N, n_nodes, n_el, n_edges;
    double *x, *w, *D;          /* LGL nodes/weights (N), D column-major N*N */
    double *xs, *ys;            /* element corner coordinates [E][4] */
    int *corner_ids;            /* [E][4] */
    /* edges (include/Edge.hpp:6-27), first-seen order */
    int *edge_type;             /* [n_edges] */
    int *edge_el;               /* [n_edges][2] */
    int *edge_side;             /* [n_edges][2], sides +-1..4 */
    int *edge_start, *edge_delta;
    /* corner nodes (include/CornerNode.hpp:8-29) */
    int *node_type;             /* [n_nodes] */
    double *node_x, *node_y;
    int *node_ptr;              /* CSR [n_nodes+1] */
    int *node_el, *node_i, *node_j;
    /* metrics (include/Quad.hpp:17-21), [E][N][N] */
    double *J, *A, *B, *C;
    /* natural boundary (no counterpart in the reference): boundary edges are
     * not masked and boundary corners assemble like interior ones */
    int neumann;
} or_mesh;

/* switch the mesh to the natural boundary */
void or_mesh_set_neumann(or_mesh* m);

/* a1: include/gauss_lobatto.hpp:43-126.  n = degree; x, w hold n+1 values.
 * Returns 0 on success. */
int or_gauss_lobatto(int n, double* x, double* w);
/* a2: include/derivative_matrix.hpp:12-38; D column-major n x n */
void or_derivative_matrix(int n, const double* x, double* D);
/* Legendre P_n and P_n' (the Boost.Math functions the reference calls) */
double or_legendre_p(int n, double x);
double or_legendre_p_prime(int n, double x);

/* a17: include/load_mesh.hpp:76-209 from in-memory arrays
 * (coords = n_nodes x 2, elements = n_el x 4 CCW corner ids). */
or_mesh* or_mesh_create(int p, int n_nodes, const double* coords, int n_el, const int* elements);
/* include/load_mesh.hpp:76-209 reading the reference's folder format */
or_mesh* or_mesh_load(int p, const char* folder);
/* a3: include/openmp_impl/Mesh.hpp:70-75, include/Quad.hpp:27-55.
 * ref_compat != 0 reproduces the reference's C(i,j) formula (Quad.hpp:53). */
void or_mesh_compute_metrics(or_mesh* m, int ref_compat);
void or_mesh_free(or_mesh* m);
/* include/openmp_impl/Mesh.hpp:84-87 */
int or_mesh_dof(const or_mesh* m);
/* include/Quad.hpp:57-62 for every node of every element: x,y [E][N][N] */
void or_mesh_node_coords(const or_mesh* m, double* x, double* y);

/* a8-a11: include/openmp_impl/{unmask,global_sum,mask,dot}.hpp */
void or_unmask(const or_mesh* m, double* a);
void or_global_sum(const or_mesh* m, double* a);
void or_mask(const or_mesh* m, double* a);
double or_dot(const or_mesh* m, const double* a, const double* b);

/* a4: include/glaplace.hpp:16-28 for one element */
void or_glaplace(const or_mesh* m, int e, const double* u, double* out);
/* a5: include/openmp_impl/galerkin.hpp:42-57 */
void or_gproj(const or_mesh* m, const double* u, double* out);
/* a7: galerkin_op of glaplace (include/openmp_impl/poisson.hpp:31-47) */
void or_apply_laplace(const or_mesh* m, const double* u, double* out);
/* a7: include/openmp_impl/helmholtz.hpp:32-52 */
void or_apply_helmholtz(const or_mesh* m, const double* c, const double* u, double* out);
/* a6: Res closure, include/openmp_impl/schrodinger.hpp:344-366 */
void or_schro_res(const or_mesh* m, const double* V, double alpha,
                  const double* q_re, const double* q_im, double* y_re, double* y_im);
/* a6: f closure, include/openmp_impl/schrodinger.hpp:322-342 */
void or_schro_f(const or_mesh* m, const double* V,
                const double* q_re, const double* q_im, double* y_re, double* y_im);

/* a13/a14: generic Krylov solvers (include/minres.hpp:19-107, include/pcg.hpp:59-97)
 * over flat vectors of length n. */
typedef void (*or_linop)(void* ctx, const double* in, double* out);
typedef double (*or_dotfn)(void* ctx, const double* a, const double* b);
typedef struct { int success; int n_iter; double residual; } or_results;
or_results or_minres(double* x, or_linop A, void* actx, const double* b, or_dotfn dot, void* dctx,
                     long n, int maxit, double tol);
or_results or_pcg(double* x, or_linop A, void* actx, const double* b, or_dotfn dot, void* dctx,
                  long n, int maxit, double tol);

/* a15 drivers */
or_results or_poisson(const or_mesh* m, double* u, const double* f, int max_iter, double tol);
or_results or_helmholtz(const or_mesh* m, double* u, const double* c, const double* f, int max_iter, double tol);
/* include/ode_base.hpp:6-13 */
typedef struct { int max_iter; double tol; double dt; int verbose; } or_solver_opts;
/* callback(user, step, psi_re, psi_im, stage_iters, n_stages) -> nonzero stops */
typedef int (*or_callback)(void* user, int step, const double* psi_re, const double* psi_im,
                           const int* stage_iters, int n_stages);
int or_schrodinger_bdf2(const or_mesh* m, double* psi_re, double* psi_im, const double* V,
                        double T, const or_solver_opts* opts, or_callback cb, void* user);
int or_schrodinger_dirk4s5(const or_mesh* m, double* psi_re, double* psi_im, const double* V,
                           double T, const or_solver_opts* opts, or_callback cb, void* user);
int or_schrodinger_dirk4s3(const or_mesh* m, double* psi_re, double* psi_im, const double* V,
                           double T, const or_solver_opts* opts, or_callback cb, void* user);

/* thread control for the CPU baseline */
void or_set_threads(int n);
int or_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
