// pixel.cuh -- warp-per-pixel phase linking for sm_103a.
//
// One warp owns one pixel and runs the whole per-pixel body of the
// reference's evd / phase_link loop (src/evd/evd.cpp:514-786,
// src/phase_link/phase_link.cpp:480-665) out of registers and a per-warp
// shared-memory slab:
//   1. SHP gather: the window is walked 32 taps at a time; the nmap bits of a
//      tap chunk are compacted with a warp ballot and the selected samples
//      (all dates) are staged in shared memory;
//   2. Gamma = sum x x^H over the SHPs, register-blocked (each lane owns an
//      BR x 4 block of the upper triangle), then normalised to coherence;
//   3. eigen-solves in shared memory: Householder tridiagonalisation, warp
//      multisection on the Sturm count, inverse iteration on the tridiagonal,
//      back-transformation; Cholesky tests and inverse for MLE;
//   4. phase referencing, compressed SLC and temporal coherence with warp
//      shuffles.
// T = float is the plain FP32 form.  Discrete decisions (eigenvalue < 1e-6,
// "is |Gamma| positive definite") whose FP32 answer lies inside a rounding
// band are not taken in FP32: the pixel is appended to a list and settled by
// the same code instantiated with T = double.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fpl {

// ------------------------------------------------------------------------
// parameters shared by all pixel kernels
// ------------------------------------------------------------------------
struct KParams {
    const float2 *__restrict__ stack;   // [nb][rows][cols]
    const uint32_t *__restrict__ nmap;  // [rows][cols][nulong]
    float2 *phase;                      // [nb][rows][cols]
    float *tcorr;                       // [rows][cols]
    float2 *comp;                       // [rows][cols]
    int32_t *status;                    // optional [rows][cols]
    long long plane;                    // rows * cols
    long long pix_begin, npix;          // first pixel, pixel count
    int rows, cols, nb, ny, nx, wx, K, nulong;
    int method, semantics, mini, bw, min_neigh;
    float amb;                          // width of the FP32 ambiguity band, in units of n*eps*|A|_F
    int *fb_count;                      // FP64 work list (scratch)
    long long *fb_list;
    int fb_cap;
    unsigned *err;                      // error flags (scratch)
};

enum { M_MLE = 0, M_EVD = 1, M_STBAS = 2 };
enum { SEM_EVD = 0, SEM_PL = 1 };
enum { ERR_FB_OVERFLOW = 1u };

// ------------------------------------------------------------------------
// complex helpers
// ------------------------------------------------------------------------
template <typename T> struct C2 { T x, y; };

template <typename T> __device__ __forceinline__ C2<T> cmk(T a, T b) { C2<T> r; r.x = a; r.y = b; return r; }
template <typename T> __device__ __forceinline__ C2<T> cadd(C2<T> a, C2<T> b) { return cmk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ C2<T> csub(C2<T> a, C2<T> b) { return cmk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ C2<T> cmul(C2<T> a, C2<T> b) { return cmk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// a * conj(b)
template <typename T> __device__ __forceinline__ C2<T> cmulc(C2<T> a, C2<T> b) { return cmk<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
// conj(a) * b
template <typename T> __device__ __forceinline__ C2<T> ccmul(C2<T> a, C2<T> b) { return cmk<T>(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x); }
template <typename T> __device__ __forceinline__ C2<T> cscale(C2<T> a, T s) { return cmk<T>(a.x * s, a.y * s); }
template <typename T> __device__ __forceinline__ T cabs2(C2<T> a) { return a.x * a.x + a.y * a.y; }
template <typename T> __device__ __forceinline__ C2<T> cconj(C2<T> a) { return cmk<T>(a.x, -a.y); }
template <typename T> __device__ __forceinline__ C2<T> cdiv(C2<T> a, C2<T> b)
{
    T den = b.x * b.x + b.y * b.y;
    return cmk<T>((a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den);
}

template <typename T> __device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <typename T> __device__ __forceinline__ T warp_max(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
template <typename T> __device__ __forceinline__ T warp_min(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <typename T> struct Eps;
template <> struct Eps<float> { static constexpr float v = 1.1920929e-7f; static constexpr float tiny = 1.17549435e-38f; };
template <> struct Eps<double> { static constexpr double v = 2.220446049250313e-16; static constexpr double tiny = 2.2250738585072014e-308; };

// ------------------------------------------------------------------------
// per-warp shared-memory slab layout
// ------------------------------------------------------------------------
__host__ __device__ constexpr size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }

template <typename T, int NP> struct Lay {
    static constexpr int LD = NP + 1;        // matrix row stride (odd: conflict-free columns)
    static constexpr int XS = NP + 2;        // staging row stride in float2 (16-byte rows)
    static constexpr size_t cm = 0;                                              // coherence C
    static constexpr size_t wm = align16(cm + sizeof(C2<T>) * NP * LD);          // work matrix / staging
    static constexpr size_t lr = align16(wm + cmax(sizeof(C2<T>) * NP * LD, sizeof(float2) * 32 * XS));
    static constexpr size_t xr = align16(lr + sizeof(T) * NP * LD);              // real work 2
    static constexpr size_t vw = align16(xr + sizeof(T) * NP * LD);              // complex vec w
    static constexpr size_t tu = align16(vw + sizeof(C2<T>) * NP);               // tau
    static constexpr size_t dd = align16(tu + sizeof(C2<T>) * NP);               // d
    static constexpr size_t ee = align16(dd + sizeof(T) * NP);                   // e
    static constexpr size_t e2 = align16(ee + sizeof(T) * NP);                   // e^2
    static constexpr size_t yy = align16(e2 + sizeof(T) * NP);                   // y / misc real vec
    static constexpr size_t ph = align16(yy + sizeof(T) * NP);                   // phases (float2)
    static constexpr size_t bytes = align16(ph + sizeof(float2) * NP);
};

// ------------------------------------------------------------------------
// warp Cholesky (lower, in place).  Returns false at the first pivot that is
// not > 0 (or NaN), like zpotrf's test (AJJ <= 0 .or. disnan(AJJ)).
// Keeps L in the lower triangle, sqrt pivots on the diagonal.
// ------------------------------------------------------------------------
template <typename T, int LD>
__device__ bool warp_chol_c(C2<T> *A, int n, int lane)
{
    for (int j = 0; j < n; ++j) {
        T piv = A[j * LD + j].x;
        if (!(piv > T(0))) return false;
        T sq = sqrt(piv);
        T r = T(1) / sq;
        __syncwarp();
        for (int i = j + 1 + lane; i < n; i += 32) A[i * LD + j] = cscale(A[i * LD + j], r);
        if (lane == 0) A[j * LD + j] = cmk<T>(sq, T(0));
        __syncwarp();
        for (int i = j + 1 + lane; i < n; i += 32) {
            C2<T> li = A[i * LD + j];
            for (int k = j + 1; k <= i; ++k) {
                C2<T> lk = A[k * LD + j];
                A[i * LD + k] = csub(A[i * LD + k], cmulc(li, lk));
            }
        }
        __syncwarp();
    }
    return true;
}

template <typename T, int LD>
__device__ bool warp_chol_r(T *A, int n, int lane)
{
    for (int j = 0; j < n; ++j) {
        T piv = A[j * LD + j];
        if (!(piv > T(0))) return false;
        T sq = sqrt(piv);
        T r = T(1) / sq;
        __syncwarp();
        for (int i = j + 1 + lane; i < n; i += 32) A[i * LD + j] *= r;
        if (lane == 0) A[j * LD + j] = sq;
        __syncwarp();
        for (int i = j + 1 + lane; i < n; i += 32) {
            T li = A[i * LD + j];
            for (int k = j + 1; k <= i; ++k) A[i * LD + k] -= li * A[k * LD + j];
        }
        __syncwarp();
    }
    return true;
}

// lambda_min(A) vs thr: +1 certainly above, -1 certainly at or below,
// 0 inside the rounding band [thr - delta, thr + delta].
template <typename T, int LD>
__device__ int lam_min_test_c(const C2<T> *A, C2<T> *W, int n, T thr, T delta, int lane)
{
    const int nsh = delta > T(0) ? 2 : 1;
    for (int s = 0; s < nsh; ++s) {
        T sh = (nsh == 1) ? thr : (s == 0 ? thr + delta : thr - delta);
        __syncwarp();
        for (int i = lane; i < n; i += 32) {
            for (int j = 0; j <= i; ++j) W[i * LD + j] = A[i * LD + j];
            W[i * LD + i].x -= sh;
        }
        __syncwarp();
        bool ok = warp_chol_c<T, LD>(W, n, lane);
        __syncwarp();
        if (nsh == 1) return ok ? 1 : -1;
        if (s == 0 && ok) return 1;
        if (s == 1 && !ok) return -1;
    }
    return 0;
}

template <typename T, int LD>
__device__ int lam_min_test_r(const T *A, T *W, int n, T thr, T delta, int lane)
{
    const int nsh = delta > T(0) ? 2 : 1;
    for (int s = 0; s < nsh; ++s) {
        T sh = (nsh == 1) ? thr : (s == 0 ? thr + delta : thr - delta);
        __syncwarp();
        for (int i = lane; i < n; i += 32) {
            for (int j = 0; j <= i; ++j) W[i * LD + j] = A[i * LD + j];
            W[i * LD + i] -= sh;
        }
        __syncwarp();
        bool ok = warp_chol_r<T, LD>(W, n, lane);
        __syncwarp();
        if (nsh == 1) return ok ? 1 : -1;
        if (s == 0 && ok) return 1;
        if (s == 1 && !ok) return -1;
    }
    return 0;
}

// inverse of a real SPD matrix from its Cholesky factor L (lower, in L):
// X = L^{-T} L^{-1}; lane j solves column j (forward then back substitution).
// X must not alias L.  Full symmetric X is written.
template <typename T, int LD>
__device__ void warp_chol_inverse_r(const T *L, T *X, int n, int lane)
{
    for (int j = lane; j < n; j += 32) {
        // forward: L y = e_j ; y_i = 0 for i < j.  y stored in X[i][j].
        for (int i = 0; i < j; ++i) X[i * LD + j] = T(0);
        for (int i = j; i < n; ++i) {
            T s = (i == j) ? T(1) : T(0);
            for (int k = j; k < i; ++k) s -= L[i * LD + k] * X[k * LD + j];
            X[i * LD + j] = s / L[i * LD + i];
        }
        // back: L^T x = y
        for (int i = n - 1; i >= 0; --i) {
            T s = X[i * LD + j];
            for (int k = i + 1; k < n; ++k) s -= L[k * LD + i] * X[k * LD + j];
            X[i * LD + j] = s / L[i * LD + i];
        }
    }
    __syncwarp();
}

// ------------------------------------------------------------------------
// Householder tridiagonalisation (restates the zhetd2/zlarfg reduction):
// Q^H A Q = T, Q = H(0)..H(n-2), reflector v_k in A[k+1.., k] (v_k[0] = 1),
// tau_k in tau, d / e real.  A is full Hermitian storage, row i on lane i%32.
// ------------------------------------------------------------------------
template <typename T, int LD>
__device__ void warp_tridiag(C2<T> *A, int n, T *d, T *e, C2<T> *tau, C2<T> *wv, int lane)
{
    for (int k = 0; k < n - 1; ++k) {
        T s = T(0);
        for (int i = k + 2 + lane; i < n; i += 32) s += cabs2(A[i * LD + k]);
        s = warp_sum(s);
        C2<T> alpha = A[(k + 1) * LD + k];
        C2<T> t = cmk<T>(T(0), T(0));
        T beta;
        if (s == T(0) && alpha.y == T(0)) {
            beta = alpha.x;
        } else {
            T nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + s);
            beta = alpha.x >= T(0) ? -nrm : nrm;
            t = cmk<T>((beta - alpha.x) / beta, -alpha.y / beta);
            C2<T> scal = cdiv(cmk<T>(T(1), T(0)), cmk<T>(alpha.x - beta, alpha.y));
            for (int i = k + 2 + lane; i < n; i += 32) A[i * LD + k] = cmul(A[i * LD + k], scal);
        }
        __syncwarp();
        if (lane == 0) {
            A[(k + 1) * LD + k] = cmk<T>(T(1), T(0));
            tau[k] = t;
            e[k] = beta;
            d[k] = A[k * LD + k].x;
        }
        __syncwarp();
        if (t.x != T(0) || t.y != T(0)) {
            // p = t * A22 v ; K = -1/2 t (p^H v) ; w = p + K v
            C2<T> p0 = cmk<T>(T(0), T(0)), p1 = cmk<T>(T(0), T(0));
            C2<T> pv = cmk<T>(T(0), T(0));
            int i0 = k + 1 + lane, i1 = i0 + 32;
            if (i0 < n) {
                C2<T> acc = cmk<T>(T(0), T(0));
                for (int j = k + 1; j < n; ++j) acc = cadd(acc, cmul(A[i0 * LD + j], A[j * LD + k]));
                p0 = cmul(t, acc);
                pv = cadd(pv, ccmul(p0, A[i0 * LD + k]));
            }
            if (i1 < n) {
                C2<T> acc = cmk<T>(T(0), T(0));
                for (int j = k + 1; j < n; ++j) acc = cadd(acc, cmul(A[i1 * LD + j], A[j * LD + k]));
                p1 = cmul(t, acc);
                pv = cadd(pv, ccmul(p1, A[i1 * LD + k]));
            }
            pv.x = warp_sum(pv.x);
            pv.y = warp_sum(pv.y);
            C2<T> K = cscale(cmul(t, pv), T(-0.5));
            if (i0 < n) wv[i0] = cadd(p0, cmul(K, A[i0 * LD + k]));
            if (i1 < n) wv[i1] = cadd(p1, cmul(K, A[i1 * LD + k]));
            __syncwarp();
            // A22 -= v w^H + w v^H
            for (int i = k + 1 + lane; i < n; i += 32) {
                C2<T> vi = A[i * LD + k], wi = wv[i];
                for (int j = k + 1; j < n; ++j) {
                    C2<T> vj = A[j * LD + k], wj = wv[j];
                    A[i * LD + j] = csub(A[i * LD + j], cadd(cmulc(vi, wj), cmulc(wi, vj)));
                }
            }
            __syncwarp();
        }
    }
    if (lane == 0) d[n - 1] = A[(n - 1) * LD + (n - 1)].x;
    __syncwarp();
}

// Sturm count: eigenvalues of T below sigma (dstebz recurrence)
template <typename T>
__device__ __forceinline__ int sturm(const T *d, const T *e2, int n, T sigma, T pivmin)
{
    int cnt = 0;
    T q = d[0] - sigma;
    if (abs(q) <= pivmin) q = -pivmin;
    cnt += q < T(0);
    for (int i = 1; i < n; ++i) {
        q = (d[i] - sigma) - e2[i - 1] / q;
        if (abs(q) <= pivmin) q = -pivmin;
        cnt += q < T(0);
    }
    return cnt;
}

// index-th (1-based ascending) eigenvalue of the tridiagonal (d, e) by
// 33-way warp multisection of the Gershgorin interval.
template <typename T>
__device__ T warp_tridiag_eig(const T *d, const T *e, T *e2, int n, int index, T *tnorm_out, int lane)
{
    T gl = T(1e30), gu = T(-1e30), em = T(0);
    for (int i = lane; i < n; i += 32) {
        T r = T(0);
        if (i > 0) r += abs(e[i - 1]);
        if (i < n - 1) { r += abs(e[i]); e2[i] = e[i] * e[i]; em = max(em, e[i] * e[i]); }
        gl = min(gl, d[i] - r);
        gu = max(gu, d[i] + r);
    }
    gl = warp_min(gl);
    gu = warp_max(gu);
    em = warp_max(em);
    __syncwarp();
    const T eps = Eps<T>::v;
    T pivmin = Eps<T>::tiny * max(T(1), em) * T(4);
    T tnorm = max(abs(gl), abs(gu));
    T fudge = T(2.1) * eps * tnorm * T(n) + T(2) * pivmin;
    T lo = gl - fudge, hi = gu + fudge;
    for (int it = 0; it < 64; ++it) {
        T tol = T(2) * eps * max(abs(lo), abs(hi)) + pivmin;
        if (hi - lo <= tol) break;
        T w = (hi - lo) / T(33);
        T sig = lo + w * T(lane + 1);
        if (lane == 31) sig = min(sig, hi);
        int c = sturm(d, e2, n, sig, pivmin);
        unsigned ge = __ballot_sync(0xffffffffu, c >= index);
        int f = ge ? (__ffs(ge) - 1) : 32;        // first point with count >= index
        T s_f = __shfl_sync(0xffffffffu, sig, f & 31);
        T s_p = __shfl_sync(0xffffffffu, sig, (f - 1) & 31);
        T nlo = (f == 0) ? lo : s_p;
        T nhi = (f == 32) ? hi : s_f;
        if (!(nhi < hi || nlo > lo)) break;       // no progress (rounding floor)
        lo = nlo;
        hi = nhi;
    }
    if (tnorm_out) *tnorm_out = tnorm;
    return T(0.5) * (lo + hi);
}

// eigenvector of the tridiagonal for eigenvalue lam: inverse iteration with
// partial pivoting (dlagtf / dlagts), run by lane 0 on shared-memory scratch
// wk (5 * n entries); the result is left in y (shared memory).
template <typename T>
__device__ void tridiag_inverse_iteration(const T *d, const T *e, int n, T lam, T tnorm, T *y,
                                          T *wk, int lane)
{
    if (lane == 0) {
        T *dg = wk, *u1 = wk + n, *u2 = wk + 2 * n, *l = wk + 3 * n, *pv = wk + 4 * n;
        const T eps = Eps<T>::v * (tnorm > T(0) ? tnorm : T(1));
        for (int i = 0; i < n; ++i) {
            dg[i] = d[i] - lam;
            u1[i] = (i < n - 1) ? e[i] : T(0);
            u2[i] = T(0);
            l[i] = T(0);
            pv[i] = T(0);
        }
        for (int i = 0; i < n - 1; ++i) {
            T sub = e[i];
            if (abs(dg[i]) >= abs(sub)) {
                if (dg[i] == T(0)) dg[i] = eps;
                l[i] = sub / dg[i];
                dg[i + 1] -= l[i] * u1[i];
            } else {
                T mult = dg[i] / sub;
                T old_u1 = u1[i];
                dg[i] = sub;
                u1[i] = dg[i + 1];
                u2[i] = (i < n - 2) ? u1[i + 1] : T(0);
                dg[i + 1] = old_u1 - mult * u1[i];
                if (i < n - 2) u1[i + 1] = -mult * u2[i];
                l[i] = mult;
                pv[i] = T(1);
            }
        }
        if (dg[n - 1] == T(0)) dg[n - 1] = eps;
        unsigned s = 12345u;
        for (int i = 0; i < n; ++i) {
            s = s * 1103515245u + 12345u;
            y[i] = T((s >> 8) & 0xFFFF) / T(65535) + T(0.5);
        }
        for (int it = 0; it < 3; ++it) {
            for (int i = 0; i < n - 1; ++i) {
                if (pv[i] != T(0)) { T t = y[i]; y[i] = y[i + 1]; y[i + 1] = t - l[i] * y[i]; }
                else y[i + 1] -= l[i] * y[i];
            }
            for (int i = n - 1; i >= 0; --i) {
                T t = y[i];
                if (i + 1 < n) t -= u1[i] * y[i + 1];
                if (i + 2 < n) t -= u2[i] * y[i + 2];
                y[i] = t / dg[i];
            }
            T mx = T(0);
            for (int i = 0; i < n; ++i) mx = max(mx, abs(y[i]));
            if (!(mx > T(0)) || !isfinite(mx)) { for (int i = 0; i < n; ++i) y[i] = T(1); continue; }
            T r = T(1) / mx;
            for (int i = 0; i < n; ++i) y[i] *= r;
        }
    }
    __syncwarp();
}

// Eigenpair of the Hermitian matrix in W (destroyed): index-th eigenvalue
// (1-based ascending).  Returns the eigenvalue; lane i gets z_i (and z_{i+32}).
template <typename T, int NP>
__device__ T warp_eigpair(C2<T> *W, int n, int index, unsigned char *sm, int lane,
                          C2<T> &z0, C2<T> &z1)
{
    using L = Lay<T, NP>;
    constexpr int LD = L::LD;
    T *d = reinterpret_cast<T *>(sm + L::dd);
    T *e = reinterpret_cast<T *>(sm + L::ee);
    T *e2 = reinterpret_cast<T *>(sm + L::e2);
    T *y = reinterpret_cast<T *>(sm + L::yy);
    T *wk = reinterpret_cast<T *>(sm + L::lr);   // free while the eigenpair is computed
    C2<T> *tau = reinterpret_cast<C2<T> *>(sm + L::tu);
    C2<T> *wv = reinterpret_cast<C2<T> *>(sm + L::vw);
    if (n == 1) {
        z0 = cmk<T>(T(1), T(0));
        z1 = cmk<T>(T(0), T(0));
        return W[0].x;
    }
    warp_tridiag<T, LD>(W, n, d, e, tau, wv, lane);
    T tnorm;
    T lam = warp_tridiag_eig<T>(d, e, e2, n, index, &tnorm, lane);
    tridiag_inverse_iteration<T>(d, e, n, lam, tnorm, y, wk, lane);
    int i0 = lane, i1 = lane + 32;
    z0 = (i0 < n) ? cmk<T>(y[i0], T(0)) : cmk<T>(T(0), T(0));
    z1 = (i1 < n) ? cmk<T>(y[i1], T(0)) : cmk<T>(T(0), T(0));
    for (int k = n - 2; k >= 0; --k) {
        C2<T> t = tau[k];
        if (t.x == T(0) && t.y == T(0)) continue;
        C2<T> s = cmk<T>(T(0), T(0));
        if (i0 >= k + 1 && i0 < n) s = cadd(s, ccmul(W[i0 * LD + k], z0));
        if (i1 >= k + 1 && i1 < n) s = cadd(s, ccmul(W[i1 * LD + k], z1));
        s.x = warp_sum(s.x);
        s.y = warp_sum(s.y);
        s = cmul(t, s);
        if (i0 >= k + 1 && i0 < n) z0 = csub(z0, cmul(s, W[i0 * LD + k]));
        if (i1 >= k + 1 && i1 < n) z1 = csub(z1, cmul(s, W[i1 * LD + k]));
    }
    return lam;
}

// ------------------------------------------------------------------------
// per-pixel driver
// ------------------------------------------------------------------------
template <typename T> struct BlockShape;
template <> struct BlockShape<float> { static constexpr int BR = 8; };
template <> struct BlockShape<double> { static constexpr int BR = 4; };

template <typename T>
__device__ __forceinline__ void acc_prod(C2<T> &acc, float2 a, float2 b);

// FP32 form: fused multiply-adds in FP32
template <>
__device__ __forceinline__ void acc_prod<float>(C2<float> &acc, float2 a, float2 b)
{
    acc.x = fmaf(a.x, b.x, fmaf(a.y, b.y, acc.x));
    acc.y = fmaf(a.y, b.x, fmaf(-a.x, b.y, acc.y));
}
// FP64 form: the reference's FP32 product, accumulated in FP64 (evd.cpp:556)
template <>
__device__ __forceinline__ void acc_prod<double>(C2<double> &acc, float2 a, float2 b)
{
    float re = __fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
    float im = __fsub_rn(__fmul_rn(a.y, b.x), __fmul_rn(a.x, b.y));
    acc.x += double(re);
    acc.y += double(im);
}

template <typename T>
__device__ __forceinline__ void defer_fp64(const KParams &P, long long pp, int lane)
{
    if (lane == 0) {
        int idx = atomicAdd(P.fb_count, 1);
        if (idx < P.fb_cap) P.fb_list[idx] = pp;
        else atomicOr(P.err, ERR_FB_OVERFLOW);
    }
}

template <typename T, int NP>
__device__ void process_pixel(const KParams &P, long long pp, unsigned char *sm, int lane)
{
    using L = Lay<T, NP>;
    constexpr int LD = L::LD;
    constexpr int XS = L::XS;
    constexpr int BR = BlockShape<T>::BR, BC = 4;
    constexpr int NBR = NP / BR, NBC = NP / BC;
    constexpr int CPR = BR / BC;   // first block column of block row R is CPR*R
    constexpr int NBLK = NBR * NBC - CPR * NBR * (NBR - 1) / 2;
    constexpr int PASSES = (NBLK + 31) / 32;

    C2<T> *Cm = reinterpret_cast<C2<T> *>(sm + L::cm);
    C2<T> *Wm = reinterpret_cast<C2<T> *>(sm + L::wm);
    float2 *Xs = reinterpret_cast<float2 *>(sm + L::wm);
    T *Lr = reinterpret_cast<T *>(sm + L::lr);
    T *Xr = reinterpret_cast<T *>(sm + L::xr);
    T *yv = reinterpret_cast<T *>(sm + L::yy);
    float2 *phs = reinterpret_cast<float2 *>(sm + L::ph);

    const int n = P.nb;
    const int cols = P.cols, rows = P.rows;
    const long long plane = P.plane;
    const uint32_t *cen = P.nmap + pp * P.nulong;
    const int cr = int(pp / cols), cc = int(pp % cols);

    // zero the outputs (the reference zeroes its block buffers, evd.cpp:447-454)
    for (int b = lane; b < n; b += 32) P.phase[b * plane + pp] = make_float2(0.f, 0.f);
    if (lane == 0) {
        P.tcorr[pp] = 0.f;
        P.comp[pp] = make_float2(0.f, 0.f);
    }
    const int cflat = P.ny * P.wx + P.nx;
    const bool centre = (__ldg(cen + (cflat >> 5)) >> (cflat & 31)) & 1u;
    if (!centre) {                                           // evd.cpp:517
        if (P.status && lane == 0) P.status[pp] = 1;
        return;
    }

    // ---- block ownership for the Gamma accumulation ----------------------
    int bR[PASSES], bC[PASSES];
    bool bAct[PASSES];
#pragma unroll
    for (int ps = 0; ps < PASSES; ++ps) {
        int b = ps * 32 + lane;
        int R = 0, rem = b;
        while (R < NBR && rem >= NBC - CPR * R) { rem -= NBC - CPR * R; ++R; }
        bR[ps] = R;
        bC[ps] = CPR * R + rem;
        bAct[ps] = (b < NBLK) && (BR * R < n) && (BC * bC[ps] < n);
    }
    C2<T> acc[BR][BC];
    if (PASSES == 1) {
#pragma unroll
        for (int i = 0; i < BR; ++i)
#pragma unroll
            for (int j = 0; j < BC; ++j) acc[i][j] = cmk<T>(T(0), T(0));
    } else {
        for (int i = lane; i < NP; i += 32)
            for (int j = 0; j < NP; ++j) Cm[i * LD + j] = cmk<T>(T(0), T(0));
        __syncwarp();
    }

    // ---- gather (ballot compaction) + accumulation (evd.cpp:539-564) -----
    int npix = 0;
    const unsigned lt = (1u << lane) - 1u;
    for (int f0 = 0; f0 < P.K; f0 += 32) {
        const int f = f0 + lane;
        bool set = false;
        long long q = 0;
        if (f < P.K) {
            int ii = f / P.wx - P.ny, jj = f % P.wx - P.nx;
            int r = cr + ii, c = cc + jj;
            if (r >= 0 && r < rows && c >= 0 && c < cols) {
                set = (__ldg(cen + (f >> 5)) >> (f & 31)) & 1u;
                q = (long long)r * cols + c;
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, set);
        const int cnt = __popc(m);
        if (cnt == 0) continue;
        __syncwarp();
        if (set) {
            const int rk = __popc(m & lt);
            const float2 *src = P.stack + q;
            float2 *dst = Xs + rk * XS;
#pragma unroll 4
            for (int t = 0; t < n; ++t) dst[t] = __ldg(src + t * plane);
        }
        __syncwarp();
        npix += cnt;
#pragma unroll
        for (int ps = 0; ps < PASSES; ++ps) {
            if (!bAct[ps]) continue;
            const int r0 = BR * bR[ps], c0 = BC * bC[ps];
            if (PASSES > 1) {
#pragma unroll
                for (int i = 0; i < BR; ++i)
#pragma unroll
                    for (int j = 0; j < BC; ++j) acc[i][j] = Cm[(r0 + i) * LD + c0 + j];
            }
            for (int s = 0; s < cnt; ++s) {
                const float2 *xs = Xs + s * XS;
                float2 xr[BR], xc[BC];
#pragma unroll
                for (int i = 0; i < BR; i += 2) {
                    float4 v = *reinterpret_cast<const float4 *>(xs + r0 + i);
                    xr[i] = make_float2(v.x, v.y);
                    xr[i + 1] = make_float2(v.z, v.w);
                }
#pragma unroll
                for (int j = 0; j < BC; j += 2) {
                    float4 v = *reinterpret_cast<const float4 *>(xs + c0 + j);
                    xc[j] = make_float2(v.x, v.y);
                    xc[j + 1] = make_float2(v.z, v.w);
                }
#pragma unroll
                for (int i = 0; i < BR; ++i)
#pragma unroll
                    for (int j = 0; j < BC; ++j) acc_prod<T>(acc[i][j], xr[i], xc[j]);
            }
            if (PASSES > 1) {
#pragma unroll
                for (int i = 0; i < BR; ++i)
#pragma unroll
                    for (int j = 0; j < BC; ++j) Cm[(r0 + i) * LD + c0 + j] = acc[i][j];
            }
        }
        __syncwarp();
    }
    if (PASSES == 1 && bAct[0]) {
        const int r0 = BR * bR[0], c0 = BC * bC[0];
#pragma unroll
        for (int i = 0; i < BR; ++i)
#pragma unroll
            for (int j = 0; j < BC; ++j) Cm[(r0 + i) * LD + c0 + j] = acc[i][j];
    }
    __syncwarp();

    const bool plink = (P.semantics == SEM_PL);
    const int min_neigh = plink ? P.min_neigh : 2;            // evd.cpp:566 / phase_link.cpp:524
    if (npix < min_neigh) {
        if (P.status && lane == 0) P.status[pp] = 2;
        return;
    }

    // ---- coherence (evd.cpp:569-582) -------------------------------------
    {
        bool bad = false;
        for (int i = lane; i < n; i += 32) {
            T Pi = Cm[i * LD + i].x;
            bad |= !(Pi > T(0)) || !isfinite(Pi);
            yv[i] = T(1) / sqrt(Pi);
        }
        bad = __any_sync(0xffffffffu, bad);
        __syncwarp();
        if (!bad) {
            for (int i = lane; i < n; i += 32) {
                const T ri = yv[i];
                for (int j = i + 1; j < n; ++j) {
                    C2<T> g = Cm[i * LD + j];
                    C2<T> c;
                    if (sizeof(T) == 8) {
                        T den = sqrt(Cm[i * LD + i].x * Cm[j * LD + j].x);
                        c = cmk<T>(g.x / den, g.y / den);
                    } else {
                        c = cscale(g, ri * yv[j]);
                    }
                    bad |= !isfinite(c.x) || !isfinite(c.y);
                    Cm[i * LD + j] = c;
                }
            }
            __syncwarp();
            for (int i = lane; i < n; i += 32) {
                for (int j = 0; j < i; ++j) Cm[i * LD + j] = cconj(Cm[j * LD + i]);
            }
            __syncwarp();
            for (int i = lane; i < n; i += 32) Cm[i * LD + i] = cmk<T>(T(1), T(0));
            bad = __any_sync(0xffffffffu, bad);
            __syncwarp();
        }
        if (bad) {
            // non-finite coherence: LAPACK's answer on NaN input is undefined;
            // the first eigen call is reported as failed.
            int code = (!plink && P.method != M_MLE) ? -6 : -1;
            if (lane == 0) {
                P.tcorr[pp] = float(code);
                if (P.status) P.status[pp] = code;
            }
            return;
        }
    }

    const T amb = T(P.amb) * T(n) * Eps<T>::v;          // 0 in the FP64 form
    const T thr = T(1.0e-6);
    int mode = 0;       // 0 = MLE eigvec of M, 1 = largest eigvec of C
    int pstatus = 0;
    const int nn = n;
    auto fro = [&](const C2<T> *A) {
        T s = T(0);
        for (int i = lane; i < nn; i += 32)
            for (int j = 0; j < nn; ++j) s += cabs2(A[i * LD + j]);
        return sqrt(warp_sum(s));
    };
    auto fill_absC = [&]() {
        for (int i = lane; i < nn; i += 32)
            for (int j = 0; j < nn; ++j)
                Lr[i * LD + j] = (i == j) ? T(1) : sqrt(cabs2(Cm[i * LD + j]));
        __syncwarp();
    };
    const bool fp32 = sizeof(T) == 4;

    if (!plink) {
        if (P.method == M_MLE) {
            // evd.cpp:598-686
            if (npix < n) {
                // fewer SHPs than dates: Gamma has rank <= npix < n, so its
                // smallest eigenvalue is 0 up to FP32 product rounding (far
                // below 1e-6): the reference reports -2.
                if (lane == 0) { P.tcorr[pp] = -2.f; if (P.status) P.status[pp] = -2; }
                return;
            }
            T dC = fp32 ? amb * fro(Cm) : T(0);
            int r = lam_min_test_c<T, LD>(Cm, Wm, n, thr, dC, lane);
            if (r == 0) { defer_fp64<T>(P, pp, lane); return; }
            if (r < 0) { if (lane == 0) { P.tcorr[pp] = -2.f; if (P.status) P.status[pp] = -2; } return; }
            fill_absC();
            T sA = T(0);
            if (fp32) {
                T s = T(0);
                for (int i = lane; i < n; i += 32)
                    for (int j = 0; j < n; ++j) s += Lr[i * LD + j] * Lr[i * LD + j];
                sA = amb * sqrt(warp_sum(s));
            }
            r = lam_min_test_r<T, LD>(Lr, Xr, n, thr, sA, lane);
            if (r == 0) { defer_fp64<T>(P, pp, lane); return; }
            if (r < 0) { if (lane == 0) { P.tcorr[pp] = -4.f; if (P.status) P.status[pp] = -4; } return; }
            // |C| is positive definite with margin: factor and invert (evd.cpp:652-664)
            if (!warp_chol_r<T, LD>(Lr, n, lane)) {
                if (fp32) { defer_fp64<T>(P, pp, lane); return; }
                if (lane == 0) { P.tcorr[pp] = -5.f; if (P.status) P.status[pp] = -5; }
                return;
            }
            warp_chol_inverse_r<T, LD>(Lr, Xr, n, lane);
            mode = 0;
        } else {
            if (P.method == M_STBAS) {                       // evd.cpp:695-706
                for (int i = lane; i < n; i += 32)
                    for (int j = 0; j < n; ++j)
                        if (j - i > P.bw || i - j > P.bw) Cm[i * LD + j] = cmk<T>(T(0), T(0));
                __syncwarp();
            }
            mode = 1;
        }
    } else {
        // phase_link.cpp:540-618: MLE if |C| is invertible, else EVD
        fill_absC();
        T sA = T(0);
        if (fp32) {
            T s = T(0);
            for (int i = lane; i < n; i += 32)
                for (int j = 0; j < n; ++j) s += Lr[i * LD + j] * Lr[i * LD + j];
            sA = amb * sqrt(warp_sum(s));
        }
        int r = lam_min_test_r<T, LD>(Lr, Xr, n, T(0), sA, lane);
        if (r == 0) { defer_fp64<T>(P, pp, lane); return; }
        if (r > 0 && warp_chol_r<T, LD>(Lr, n, lane)) {
            warp_chol_inverse_r<T, LD>(Lr, Xr, n, lane);
            mode = 0;
        } else {
            mode = 1;
            pstatus = 3;
        }
    }

    // ---- the eigenvector --------------------------------------------------
    C2<T> z0, z1;
    if (mode == 0) {
        // M = inv(|C|) o C (evd.cpp:667) ; smallest eigenpair (evd.cpp:670-686)
        for (int i = lane; i < n; i += 32)
            for (int j = 0; j < n; ++j) Wm[i * LD + j] = cscale(Cm[i * LD + j], Xr[i * LD + j]);
        __syncwarp();
        T dM = T(0);
        if (fp32 && !plink) dM = amb * fro(Wm);
        __syncwarp();
        T lam = warp_eigpair<T, NP>(Wm, n, 1, sm, lane, z0, z1);
        if (!plink) {
            if (lam < thr + dM && lam >= thr - dM && fp32) { defer_fp64<T>(P, pp, lane); return; }
            if (lam < thr) { if (lane == 0) { P.tcorr[pp] = -7.f; if (P.status) P.status[pp] = -7; } return; }
        }
    } else {
        for (int i = lane; i < n; i += 32)
            for (int j = 0; j < n; ++j) Wm[i * LD + j] = Cm[i * LD + j];
        __syncwarp();
        T lam = warp_eigpair<T, NP>(Wm, n, n, sm, lane, z0, z1);
        if (!plink && lam < thr) {                           // evd.cpp:718-726
            if (lane == 0) { P.tcorr[pp] = -7.f; if (P.status) P.status[pp] = -7; }
            return;
        }
    }

    // ---- phase referencing (evd.cpp:738-749) ------------------------------
    const int mref = P.mini - 1;
    C2<T> zr;
    {
        C2<T> a = (mref < 32) ? z0 : z1;
        zr.x = __shfl_sync(0xffffffffu, a.x, mref & 31);
        zr.y = __shfl_sync(0xffffffffu, a.y, mref & 31);
    }
    const T zra = sqrt(cabs2(zr));
    const C2<T> zru = (zra > T(0)) ? cscale(zr, T(1) / zra) : cmk<T>(T(1), T(0));
    float2 ph0 = make_float2(0.f, 0.f), ph1 = make_float2(0.f, 0.f);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int i = lane + 32 * h;
        if (i >= n) continue;
        C2<T> z = h ? z1 : z0;
        T za = sqrt(cabs2(z));
        C2<T> u = (za > T(0)) ? cscale(z, T(1) / za) : cmk<T>(T(1), T(0));
        C2<T> pr = cmulc(u, zru);                       // exp(i(arg z_i - arg z_ref))
        float2 o = (i == mref) ? make_float2(1.f, 0.f) : make_float2(float(pr.x), float(pr.y));
        if (h) ph1 = o; else ph0 = o;
        phs[i] = o;
        P.phase[i * plane + pp] = o;
    }
    __syncwarp();

    // ---- compressed SLC (evd.cpp:752-762) ---------------------------------
    {
        T sr = T(0), si = T(0);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int i = lane + 32 * h;
            if (i >= n || i < mref) continue;
            float2 x = __ldg(P.stack + i * plane + pp);
            float2 o = h ? ph1 : ph0;
            float re = __fadd_rn(__fmul_rn(x.x, o.x), __fmul_rn(x.y, o.y));
            float im = __fsub_rn(__fmul_rn(x.y, o.x), __fmul_rn(x.x, o.y));
            sr += T(re);
            si += T(im);
        }
        sr = warp_sum(sr);
        si = warp_sum(si);
        if (lane == 0) {
            const T den = T(n - mref);
            P.comp[pp] = make_float2(float(sr / den), float(si / den));
        }
    }

    // ---- temporal coherence (evd.cpp:768-786) -----------------------------
    {
        const bool stbas = (P.method == M_STBAS);
        T sr = T(0), si = T(0);
        int cnt = 0;
        for (int i = lane; i < n; i += 32) {
            int ulim = stbas ? min(i + P.bw + 1, n) : n;
            const float2 pi = phs[i];
            const C2<T> cpi = cmk<T>(T(pi.x), T(pi.y));
            for (int j = i + 1; j < ulim; ++j) {
                C2<T> c = Cm[i * LD + j];
                T ca = sqrt(cabs2(c));
                C2<T> u = (ca > T(0)) ? cscale(c, T(1) / ca) : cmk<T>(T(1), T(0));
                const float2 pj = phs[j];
                // exp(i(arg C_ij - arg ph_i + arg ph_j))
                C2<T> v = cmul(cmulc(u, cpi), cmk<T>(T(pj.x), T(pj.y)));
                sr += v.x;
                si += v.y;
                cnt++;
            }
        }
        sr = warp_sum(sr);
        si = warp_sum(si);
        cnt = warp_sum(cnt);
        if (lane == 0) {
            P.tcorr[pp] = float(sqrt(sr * sr + si * si) / T(cnt));   // 0/0 = NaN for one date, as the reference
            if (P.status) P.status[pp] = pstatus;
        }
    }
}

}  // namespace fpl
