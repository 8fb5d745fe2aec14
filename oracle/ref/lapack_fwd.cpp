// Forwarders for the two LAPACK routines the reference declares
// (dsteqr_/ssteqr_, include/gauss_lobatto.hpp:22-25; it calls dsteqr for the
// quadrature of degree p > 8).  No system LAPACK is installed, so the calls
// go to a LAPACK shared library opened at run time that exports the routine
// under its own name or with a "scipy_" prefix (the OpenBLAS that SciPy
// bundles).  The library is the one given to sem_ref_lapack_open, else the
// one named by the environment variable SEM_REF_LAPACK on first use.  The
// hidden Fortran length of the character argument is passed explicitly.
//
// TEST INFRASTRUCTURE ONLY (backs the CPU reference build).
#include <dlfcn.h>

#include <cstddef>
#include <cstdio>
#include <cstdlib>

typedef void (*steqr_d_fn)(char*, int*, double*, double*, double*, int*, double*, int*, size_t);
typedef void (*steqr_s_fn)(char*, int*, float*, float*, float*, int*, float*, int*, size_t);
static steqr_d_fn g_dsteqr = nullptr;
static steqr_s_fn g_ssteqr = nullptr;

extern "C" int sem_ref_lapack_open(const char* path, char* err, int errlen)
{
    void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h)
    {
        if (err) std::snprintf(err, errlen, "%s", dlerror());
        return -1;
    }
    g_dsteqr = (steqr_d_fn)dlsym(h, "scipy_dsteqr_");
    if (!g_dsteqr) g_dsteqr = (steqr_d_fn)dlsym(h, "dsteqr_");
    g_ssteqr = (steqr_s_fn)dlsym(h, "scipy_ssteqr_");
    if (!g_ssteqr) g_ssteqr = (steqr_s_fn)dlsym(h, "ssteqr_");
    if (!g_dsteqr)
    {
        if (err) std::snprintf(err, errlen, "no dsteqr in %s", path);
        return -1;
    }
    return 0;
}

static void lazy_open()
{
    if (g_dsteqr) return;
    const char* p = std::getenv("SEM_REF_LAPACK");
    if (p) sem_ref_lapack_open(p, nullptr, 0);
}

// info = -1000 when no LAPACK is available: the reference then reports
// "eigenvalue decomposition failed"
extern "C" int dsteqr_(char* compz, int* n, double* d, double* e, double* z, int* ldz, double* work, int* info)
{
    lazy_open();
    if (!g_dsteqr)
        *info = -1000;
    else
        g_dsteqr(compz, n, d, e, z, ldz, work, info, 1);
    return 0;
}

extern "C" int ssteqr_(char* compz, int* n, float* d, float* e, float* z, int* ldz, float* work, int* info)
{
    lazy_open();
    if (!g_ssteqr)
        *info = -1000;
    else
        g_ssteqr(compz, n, d, e, z, ldz, work, info, 1);
    return 0;
}
