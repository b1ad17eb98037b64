/*
 * ref_backend.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Adapter that lets the oracle's per-pixel loop (fpl_oracle.c, built with
 * -DFPL_BACKEND_REF) call the reference's own, unmodified EVWorker
 * (include/fringe/EigenLapack.hpp:60-251), which in turn calls LAPACK
 * zheevr / zpotrf / zpotri, and the nmap oracle call the reference's own
 * two-sample KS test (src/nmap/KS2sample.hpp:96-144).  The headers are
 * compiled where they lie in the reference tree (see build_ref.sh); nothing
 * from them is copied here.
 */
#include <complex>
#include <cstring>

#include "fringe/EigenLapack.hpp"
#include "KS2sample.hpp"

extern "C" {

void *fpl_ref_ws_create(int n) { return new EVWorker(n); }

void fpl_ref_ws_destroy(void *w) { delete static_cast<EVWorker *>(w); }

int fpl_ref_ws_eig(void *w, double *A, int index, int want_vec, double *val,
                   double *vec)
{
    EVWorker *ev = static_cast<EVWorker *>(w);
    int info = ev->eigenWithIndex(reinterpret_cast<std::complex<double> *>(A),
                                  index, want_vec != 0);
    val[0] = ev->eigval[0];
    if (want_vec)
        std::memcpy(vec, ev->eigvec, sizeof(std::complex<double>) * ev->size);
    return info;
}

int fpl_ref_ws_pdinv(void *w, double *A)
{
    EVWorker *ev = static_cast<EVWorker *>(w);
    return ev->positiveDefiniteInverse(reinterpret_cast<std::complex<double> *>(A));
}

double fpl_ref_ks2(int n, const float *a, const float *b)
{
    KS2sample ks(n);
    return ks.test(a, b);
}

}
