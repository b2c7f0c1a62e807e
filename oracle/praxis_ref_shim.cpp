// ORACLE shim (test infrastructure only): exposes the reference's own PRAXIS
// (CUDA/praxis.cpp, compiled from the reference checkout by
// oracle/build_ref.py into oracle/_ref/) through a C entry point that takes a
// callback, so tests can compare it with the library's PRAXIS on the same
// functions.  praxis.hpp declares: double praxis(double t0, double h0, int n,
// int prin, double x[], double f(double x[], int n)).
#include <cstddef>
double praxis(double t0, double h0, int n, int prin, double x[], double f(double x[], int n));

typedef double (*cb_t)(const double* x, int n, void* user);
static cb_t g_cb = nullptr;
static void* g_user = nullptr;
static int g_nf = 0;
static double tramp(double x[], int n) { ++g_nf; return g_cb(x, n, g_user); }

extern "C" double ref_praxis(cb_t f, void* user, int n, double* x, double t0, double h0, int* nf) {
    g_cb = f; g_user = user; g_nf = 0;
    double v = praxis(t0, h0, n, 0, x, tramp);
    if (nf) *nf = g_nf;
    return v;
}
