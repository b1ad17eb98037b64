/*
 * ref_backend.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Adapter that lets the oracle's per-pixel loop (fpl_oracle.c, built with
 * -DFPL_BACKEND_REF) call the reference's own, unmodified EVWorker
 * (include/fringe/EigenLapack.hpp:60-251), which in turn calls LAPACK
 * zheevr / zpotrf / zpotri, and the nmap oracle call the reference's own
 * two-sample KS and Anderson-Darling tests (src/nmap/KS2sample.hpp:96-144,
 * src/nmap/AD2unique.hpp:270-347).  The headers are
 * compiled where they lie in the reference tree (see build_ref.sh); nothing
 * from them is copied here.
 */
#include <complex>
#include <cstring>

#include "fringe/EigenLapack.hpp"
#include "KS2sample.hpp"
#include "AD2unique.hpp"

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

// one test object per thread and stack depth (its constructor sums the
// harmonic series of the variance, O(n^2))
double fpl_ref_ad2(int n, const float *a, const float *b)
{
    static thread_local AD2unique *ad = nullptr;
    static thread_local int ad_n = -1;
    if (ad_n != n) {
        delete ad;
        ad = new AD2unique(n);
        ad_n = n;
    }
    return ad->test(a, b);
}

}
