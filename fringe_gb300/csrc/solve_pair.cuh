// solve_pair.cuh -- the mixed form's eigen-solve at <= 16 dates with two
// pixels per warp.
//
// A warp that solves one pixel of at most 16 dates leaves lanes 16..31
// without a row.  Here half h of the warp (lanes 16h .. 16h+15) solves one
// pixel, lane l of the half owning row l, so every instruction of the warp
// advances two pixels.  The two per-pixel slabs of 16 dates take no more
// shared memory than a CTA of one-pixel warps can hold, so a CTA keeps its
// 20 warps and holds twice the pixels.  The decisions, bands and codes are
// those of pixel_solve for the MLE method with evd semantics
// (evd.cpp:598-686), and each row's arithmetic is the same as there; only the
// sums across lanes run over 16 lanes instead of 32.
//
// Shared-memory and register work runs per half (its own slab, the masks of
// its 16 lanes).  The coherence rows live in tensor memory (the row layout of
// CRowsTmem<16>, so lane 16h + l holds row l of its half's pixel); their
// loads and stores are warp-wide instructions, so every stage that reads them
// is entered by both halves together, and a half with nothing to do there
// only takes part in the loads.  The Householder fall-back runs on the whole
// warp, one pixel at a time, as in pixel_solve; so does every pixel of
// another method or semantics (pixel_solve itself).
#pragma once
#include "pixel.cuh"

namespace fpl {
// internal linkage: the header is compiled into more than one unit
namespace {

constexpr int PNP = 16;                 // padded dates of the paired solve
using PLay = Lay<float, PNP>;
using PairRows = CRowsTmem<PNP>;

// lanes of one half
struct PairHalf {
    int hl;          // lane within the half, 0..15: the row it owns
    int h;           // which half
    unsigned hm;     // the half's lanes
};

__device__ __forceinline__ float hsum(float v, unsigned hm)
{
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) v += __shfl_xor_sync(hm, v, o, 16);
    return v;
}
__device__ __forceinline__ float hmax(float v, unsigned hm)
{
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(hm, v, o, 16));
    return v;
}
__device__ __forceinline__ C2<float> hbcast(C2<float> v, int src, unsigned hm)
{
    return cmk<float>(__shfl_sync(hm, v.x, src, 16), __shfl_sync(hm, v.y, src, 16));
}

// L2 prefetch of a pixel's Gamma record by the 16 lanes of its half
__device__ __forceinline__ void pair_prefetch(const KParams &P, long long pp, int hl)
{
    const long long loc = pp - P.cbase;
    const char *rec = reinterpret_cast<const char *>(P.cbuf) + loc * (long long)P.cstride * 4;
    const uintptr_t lo = reinterpret_cast<uintptr_t>(rec) & ~uintptr_t(127);
    const uintptr_t hi = reinterpret_cast<uintptr_t>(rec) + (size_t)P.cstride * 4;
    for (uintptr_t a = lo + 128u * (unsigned)hl; a < hi; a += 16u * 128u) asm volatile("prefetch.L2 [%0];" :: "l"(a));
    if (hl == 15) asm volatile("prefetch.L2 [%0];" :: "l"(P.cinfo + loc));
}

// Gamma record of pixel pp into G (upper triangle and diagonal), as
// pixel_load_gamma with the 16 lanes of a half.  Returns the SHP count, or
// -1 when the pixel is finished (outputs written or handed to FP64).
__device__ __forceinline__ int pair_load(const KParams &P, long long pp, C2<float> *G, const PairHalf &H)
{
    constexpr int LD = PLay::LD;
    const int n = P.nb;
    const long long plane = P.plane;
    if (H.hl < n) P.phase[H.hl * plane + pp] = make_float2(0.f, 0.f);
    if (H.hl == 0) {
        P.tcorr[pp] = 0.f;
        P.comp[pp] = make_float2(0.f, 0.f);
    }
    const long long loc = pp - P.cbase;
    const int info = P.cinfo[loc];
    if (info == CI_CENTRE || info == CI_FEW) {
        if (P.status && H.hl == 0) P.status[pp] = (info == CI_CENTRE) ? 1 : 2;
        return -1;
    }
    if (info == CI_DEFER) {
        defer_fp64(P, pp, H.hl);
        return -1;
    }
    const float4 *rec4 =
        reinterpret_cast<const float4 *>(reinterpret_cast<const float *>(P.cbuf) + loc * (long long)P.cstride);
    const int dp = (n + 1) >> 1, nblk = dp * (dp + 1) / 2;
    for (int t0 = 0; t0 < nblk; t0 += 64) {
        float4 u[4], v[4];
#pragma unroll
        for (int s4 = 0; s4 < 4; ++s4) {
            const int t = t0 + H.hl + 16 * s4;
            u[s4] = v[s4] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (t < nblk) {
                u[s4] = __ldg(rec4 + 2 * t);
                v[s4] = __ldg(rec4 + 2 * t + 1);
            }
        }
#pragma unroll
        for (int s4 = 0; s4 < 4; ++s4) {
            const int t = t0 + H.hl + 16 * s4;
            if (t >= nblk) continue;
            const int tr = nblk - 1 - t;
            const int r = (int)((sqrtf((float)(8 * tr + 1)) - 1.f) * 0.5f);
            const int a = dp - 1 - r, b = dp - 1 - (tr - r * (r + 1) / 2);
            const int i0 = 2 * a, i1 = 2 * a + 1, j0 = 2 * b, j1 = 2 * b + 1;
            if (j0 < n) G[i0 * LD + j0] = cmk<float>(u[s4].x, u[s4].y);
            if (j1 < n) G[i0 * LD + j1] = cmk<float>(u[s4].z, u[s4].w);
            if (i1 < n && j0 >= i1) G[i1 * LD + j0] = cmk<float>(v[s4].x, v[s4].y);
            if (j1 < n) G[i1 * LD + j1] = cmk<float>(v[s4].z, v[s4].w);
        }
    }
    __syncwarp(H.hm);
    return info;
}

// Gamma in G to the coherence rows (rows_coherence on 16 lanes).  Every lane
// of the warp calls it; go: this half holds a record in G.  Returns false
// unless go and every value is finite (the code is written then);
// *cfro = |C|_F.
__device__ __forceinline__ bool pair_coherence(const KParams &P, long long pp, const C2<float> *G, unsigned char *sm,
                                               const PairRows &cp, const PairHalf &H, bool go, float *cfro)
{
    constexpr int LD = PLay::LD;
    float *yv = reinterpret_cast<float *>(sm + PLay::yy);
    const int n = go ? P.nb : 0;
    const int i = H.hl;
    bool bad = false;
    if (i < n) {
        const float Pi = G[i * LD + i].x;
        bad = !(Pi > 0.f) || !isfinite(Pi);
        yv[i] = 1.f / sqrtf(Pi);
    }
    bad = __any_sync(H.hm, bad);
    __syncwarp();
    float fs = 0.f;
    const float ri = (i < n) ? yv[i] : 0.f;
#pragma unroll 1
    for (int c = 0; c < PNP / 8; ++c) {
        const float4 ya = *reinterpret_cast<const float4 *>(yv + 8 * c);
        const float4 yb = *reinterpret_cast<const float4 *>(yv + 8 * c + 4);
        const float yj[8] = {ya.x, ya.y, ya.z, ya.w, yb.x, yb.y, yb.z, yb.w};
        C2<float> v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = 8 * c + k;
            C2<float> e = cmk<float>(0.f, 0.f);
            if (!bad && i < n && j < n) {
                if (j > i) e = cscale(G[i * LD + j], ri * yj[k]);
                else if (j < i) e = cconj(cscale(G[j * LD + i], yj[k] * ri));
                else e = cmk<float>(1.f, 0.f);
                bad |= !isfinite(e.x) || !isfinite(e.y);
                fs += cabs2(e);
            }
            v[k] = e;
        }
        cp.store(0, c, v);
    }
    cp.fence();
    bad = __any_sync(H.hm, bad);
    *cfro = sqrtf(hsum(fs, H.hm));
    __syncwarp();
    if (go && bad) put_code(P, pp, H.hl, -1);
    return go && !bad;
}

// the coherence rows into the work matrix W (full rows); every lane calls it
__device__ __forceinline__ void pair_copy_rows(const PairRows &cp, C2<float> *W, const PairHalf &H, bool go)
{
    constexpr int LD = PLay::LD;
    __syncwarp();
#pragma unroll
    for (int c = 0; c < PNP / 8; ++c) {
        C2<float> v[8];
        cp.load(0, c, v);
        if (go) {
#pragma unroll
            for (int k = 0; k < 8; ++k) W[H.hl * LD + 8 * c + k] = v[k];
        }
    }
    __syncwarp();
}

// Cholesky of the complex Hermitian A in place: warp_chol_c2 on the 16
// lanes of a half (two elimination steps per pass, the same pivot tests, and
// with STORE the same factor layout).  col: 2 x 16 complex of the half's slab.
template <bool STORE>
__device__ bool pair_chol(C2<float> *A, int n, C2<float> *col, const PairHalf &H)
{
    constexpr int LD = PLay::LD;
    C2<float> *cA = col, *cB = col + PNP;
    const int i = H.hl;
    C2<float> *Ai = A + i * LD;
    const bool row = i < n;
    for (int j = 0; j < n; j += 2) {
        const bool two = (j + 1 < n);
        const float p1 = A[j * LD + j].x;
        if (!(p1 > 0.f)) return false;
        const float r1 = rsqrtf(p1);
        const bool b1 = row && i > j;
        C2<float> l1 = cmk<float>(0.f, 0.f);
        if (b1) {
            const C2<float> a = Ai[j];
            l1 = cmk<float>(a.x * r1, a.y * r1);
        }
        float r2 = 0.f;
        C2<float> l2 = cmk<float>(0.f, 0.f);
        const bool b2 = row && i > j + 1;
        if (two) {
            const C2<float> ln = hbcast(l1, j + 1, H.hm);
            const float p2 = fmaf(-ln.y, ln.y, fmaf(-ln.x, ln.x, A[(j + 1) * LD + j + 1].x));
            if (!(p2 > 0.f)) return false;
            r2 = rsqrtf(p2);
            if (b2) {
                C2<float> a = Ai[j + 1];
                a.x = fmaf(-l1.x, ln.x, fmaf(-l1.y, ln.y, a.x));
                a.y = fmaf(-l1.y, ln.x, fmaf(l1.x, ln.y, a.y));
                l2 = cmk<float>(a.x * r2, a.y * r2);
            }
        }
        cA[i] = l1;
        cB[i] = l2;
        if (STORE) {
            if (i == j) Ai[j] = cmk<float>(r1, 0.f);
            else if (b1) Ai[j] = l1;
            if (two) {
                if (i == j + 1) Ai[j + 1] = cmk<float>(r2, 0.f);
                else if (b2) Ai[j + 1] = l2;
            }
        }
        __syncwarp(H.hm);
        if (b2) {
            // a_ik -= l1_i conj(l1_k) + l2_i conj(l2_k), k in (j+1, i]
            for (int k0 = j + 2; k0 <= i; k0 += 2) {
                const float4 a0 = *reinterpret_cast<const float4 *>(cA + k0);
                const float4 c0 = *reinterpret_cast<const float4 *>(cB + k0);
                const float la[4] = {a0.x, a0.y, a0.z, a0.w};
                const float lb[4] = {c0.x, c0.y, c0.z, c0.w};
                C2<float> x[2];
#pragma unroll
                for (int u = 0; u < 2; ++u) x[u] = Ai[k0 + u];
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const float ax = la[2 * u], ay = la[2 * u + 1], bx = lb[2 * u], by = lb[2 * u + 1];
                    x[u].x = fmaf(-l1.x, ax, x[u].x);
                    x[u].x = fmaf(-l1.y, ay, x[u].x);
                    x[u].x = fmaf(-l2.x, bx, x[u].x);
                    x[u].x = fmaf(-l2.y, by, x[u].x);
                    x[u].y = fmaf(-l1.y, ax, x[u].y);
                    x[u].y = fmaf(l1.x, ay, x[u].y);
                    x[u].y = fmaf(-l2.y, bx, x[u].y);
                    x[u].y = fmaf(l2.x, by, x[u].y);
                }
#pragma unroll
                for (int u = 0; u < 2; ++u) Ai[k0 + u] = x[u];
            }
        }
        __syncwarp(H.hm);
    }
    return true;
}

// the factor of pair_chol<true> into strict-lower form (chol_strict_lower)
__device__ __forceinline__ float pair_strict_lower(C2<float> *L, int n, const PairHalf &H)
{
    constexpr int LD = PLay::LD;
    const int i = H.hl;
    float d = 0.f;
    if (i < n) {
        C2<float> *Li = L + i * LD;
        d = Li[i].x;
        for (int k = i; k < n; ++k) Li[k] = cmk<float>(0.f, 0.f);
    }
    __syncwarp(H.hm);
    return d;
}

// (L L^H) x = b for the strict-lower factor (warp_chol_solve); b is the
// lane's row
__device__ __forceinline__ void pair_chol_solve(const C2<float> *L, int n, float d, C2<float> &b, const PairHalf &H)
{
    constexpr int LD = PLay::LD;
    const int i = H.hl;
    const C2<float> *Li = L + i * LD;
#pragma unroll 2
    for (int j = 0; j < n; ++j) {
        const C2<float> y = hbcast(cscale(b, d), j, H.hm);
        fms_mul(b, Li[j], y);
    }
    b = cscale(b, d);
#pragma unroll 2
    for (int j = n - 1; j >= 0; --j) {
        const C2<float> x = hbcast(cscale(b, d), j, H.hm);
        fms_cmul(b, L[j * LD + i], x);
    }
    b = (i < n) ? cscale(b, d) : cmk<float>(0.f, 0.f);
}

// y = A x for the Hermitian A in shared memory (warp_matvec on 16 lanes)
__device__ __forceinline__ C2<float> pair_matvec(const C2<float> *A, int n, const C2<float> *xv, const PairHalf &H)
{
    constexpr int LD = PLay::LD;
    const int i = H.hl;
    C2<float> u = cmk<float>(0.f, 0.f);
    if (i < n) {
        const C2<float> *Ai = A + i * LD;
        C2<float> a0 = cmk<float>(0.f, 0.f), a1 = cmk<float>(0.f, 0.f);
#pragma unroll 2
        for (int j = 0; j < n; j += 2) {
            const float4 q = *reinterpret_cast<const float4 *>(xv + j);
            cfma(a0, Ai[j], cmk<float>(q.x, q.y));
            if (j + 1 < n) cfma(a1, Ai[j + 1], cmk<float>(q.z, q.w));
        }
        u = cadd(a0, a1);
    }
    return u;
}

// |C| not positive definite, proved from a failed sweep: abs_not_pd on the
// 16 lanes of a half (v = (-w, 1, 0, ..) from row k of the sweep, its
// quadratic form below minus the rounding and spectral bands, refined by up
// to kNotPdSteps power steps on ||C||_inf I - |C| when it falls short).
// Every lane calls it (the rows are read from tensor memory, so the steps
// run while either half still needs one); go: this half's sweep stopped at
// step k with row k in rk.  ub: the half's 16 entries of scratch.
__device__ __forceinline__ bool pair_not_pd(const PairRows &cp, const float *rk, int k, int n, float amb,
                                            float *ub, const PairHalf &H, bool go)
{
    const int i = H.hl;
    if (go) ub[i] = (i < k) ? -rk[i] : (i == k ? 1.f : 0.f);
    const float g = float(2 * (n + 1)) * Eps<float>::v;
    float band = 0.f, anorm = 0.f;
    bool proved = false, pend = go;
    for (int it = 0;; ++it) {
        __syncwarp();
        const bool row = pend && i < n;
        const float vi = row ? ub[i] : 0.f;
        float yq = 0.f, ys = 0.f, rs = 0.f, f2 = 0.f;
#pragma unroll
        for (int c = 0; c < PNP / 8; ++c) {
            C2<float> v[8];
            cp.load(0, c, v);
#pragma unroll
            for (int kk = 0; kk < 8; ++kk) {
                const int j = 8 * c + kk;
                if (!row || j >= n) continue;
                const float m2 = cabs2(v[kk]);
                f2 += m2;
                const float a = (i == j) ? 1.f : m2 * rsqrtf(max(m2, 1e-37f));
                const float vj = ub[j];
                yq = fmaf(a, vj, yq);
                ys = fmaf(a, fabsf(vj), ys);
                rs += a;
            }
        }
        const float q = hsum(vi * yq, H.hm);
        const float sa = hsum(fabsf(vi) * ys, H.hm);
        const float v2 = hsum(vi * vi, H.hm);
        if (it == 0) {
            band = amb * sqrtf(hsum(f2, H.hm));
            anorm = hmax(rs, H.hm);
        }
        if (pend && q < -(g * sa + band * v2)) {
            proved = true;
            pend = false;
        }
        if (it == kNotPdSteps || !__any_sync(0xffffffffu, pend)) break;
        // v <- ||C||_inf v - |C| v, scaled by its largest entry
        const float u = (pend && i < n) ? fmaf(anorm, vi, -yq) : 0.f;
        const float um = hmax(fabsf(u), H.hm);
        if (!(um > 0.f)) pend = false;
        __syncwarp();
        if (pend && i < n) ub[i] = u * (1.f / um);
    }
    __syncwarp();
    return proved;
}

// |C| from the coherence rows, its symmetric sweep inverse
// (warp_sweep_inverse_rows on 16 lanes) and M = inv|C| o C into W
// (evd.cpp:623-667).  Every lane calls it; go: this half builds M.  Returns
// 1 when M is in W: every sweep pivot is > 0, cond_inf(|C|) <= cond_max and
// 1 / |inv|C||_inf > lim (which settles the lambda_min(|C|) test); -1 when a
// pivot <= 0 proves |C| not positive definite (pair_not_pd); 0 when the
// pixel goes to the FP64 path.  amb: the rounding band per unit of ||C||_F.
__device__ __forceinline__ int pair_build_M(const PairRows &cp, unsigned char *sm, C2<float> *W, const PairHalf &H,
                                            bool go, int n, float cond_max, float lim, float amb, float *xnorm)
{
    constexpr int LD = PLay::LD;
    const int i = H.hl;
    float x[PNP];
    __syncwarp();
    float rs = 0.f;
#pragma unroll
    for (int c = 0; c < PNP / 8; ++c) {
        C2<float> v[8];
        cp.load(0, c, v);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = 8 * c + k;
            const float m2 = cabs2(v[k]);
            const float a = (i == j) ? 1.f : m2 * rsqrtf(max(m2, 1e-37f));
            const bool in = go && i < n && j < n;
            x[j] = in ? a : 0.f;
            rs += in ? a : 0.f;
        }
    }
    const float anorm = hmax(rs, H.hm);
    bool ok = go;
    int kfail = -1;
    float *rowb = reinterpret_cast<float *>(sm + PLay::wk);
    if (ok) {
        // lane k publishes row k with its k-th entry replaced by p - 1 (see
        // warp_sweep_inverse_rows)
#pragma unroll 1
        for (int k = 0; k < n; ++k) {
            float *rk = rowb + (k & 1) * PNP;
            float *pk = rowb + 2 * PNP + (k & 1);
            if (i == k) {
#pragma unroll
                for (int j = 0; j < PNP; j += 4) *reinterpret_cast<float4 *>(rk + j) = make_float4(x[j], x[j + 1], x[j + 2], x[j + 3]);
                const float v = rk[k];
                *pk = v;
                rk[k] = v - 1.f;
            }
            __syncwarp(H.hm);
            const float p = *pk;
            if (!(p > 0.f)) {
                ok = false;
                kfail = k;
                break;
            }
            const float rp = 1.f / p;
            const float bm = (i == k) ? rp - 1.f : -(rk[i] * rp);
#pragma unroll
            for (int j = 0; j < PNP; j += 4) {
                const float4 r = *reinterpret_cast<const float4 *>(rk + j);
                x[j] = fmaf(bm, r.x, x[j]);
                x[j + 1] = fmaf(bm, r.y, x[j + 1]);
                x[j + 2] = fmaf(bm, r.z, x[j + 2]);
                x[j + 3] = fmaf(bm, r.w, x[j + 3]);
            }
        }
        __syncwarp(H.hm);
    }
    if (ok) {
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < PNP; ++j) {
            const float v = (j == i) ? 2.f - x[j] : -x[j];
            x[j] = v;
            if (i < n && j < n) s += fabsf(v);
        }
        *xnorm = hmax(s, H.hm);
        ok = anorm * (*xnorm) <= cond_max && 1.f / *xnorm > lim;
    }
    const bool failed = kfail >= 0;
    bool not_pd = false;
    if (__any_sync(0xffffffffu, failed))
        not_pd = pair_not_pd(cp, rowb + (kfail & 1) * PNP, kfail, n, amb, rowb + 3 * PNP, H, failed);
    // M = inv|C| o C
    __syncwarp();
#pragma unroll
    for (int c = 0; c < PNP / 8; ++c) {
        C2<float> v[8];
        cp.load(0, c, v);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = 8 * c + k;
            if (ok && i < n && j < n) W[i * LD + j] = cscale(v[k], x[j]);
        }
    }
    __syncwarp();
    return ok ? 1 : (not_pd ? -1 : 0);
}

// kPowerStartIters power iterations on C from the all-ones vector (warp_power_start);
// every lane calls it.  The unit vector comes back in z and in vv.
__device__ __forceinline__ C2<float> pair_power_start(const PairRows &cp, int n, unsigned char *sm,
                                                      const PairHalf &H)
{
    C2<float> *vv = reinterpret_cast<C2<float> *>(sm + PLay::vv);
    const int i = H.hl;
    vv[i] = cmk<float>(i < n ? 1.f : 0.f, 0.f);
    __syncwarp();
    C2<float> z = cmk<float>(0.f, 0.f);
    for (int it = 0; it < kPowerStartIters; ++it) {
        C2<float> a = cmk<float>(0.f, 0.f);
#pragma unroll 1
        for (int c = 0; c < PNP / 8; ++c) {
            C2<float> v[8];
            cp.load(0, c, v);
#pragma unroll
            for (int k = 0; k < 8; k += 2) {
                const int j = 8 * c + k;
                const float4 q = *reinterpret_cast<const float4 *>(vv + j);
                if (j < n) cfma(a, v[k], cmk<float>(q.x, q.y));
                if (j + 1 < n) cfma(a, v[k + 1], cmk<float>(q.z, q.w));
            }
        }
        const C2<float> u = (i < n) ? a : cmk<float>(0.f, 0.f);
        const float inv = rsqrtf(hsum(cabs2(u), H.hm));
        z = cscale(u, inv);
        __syncwarp();
        if (i < n) vv[i] = z;
        __syncwarp();
    }
    return z;
}

// inverse iteration on M - sigma I (warp_inverse_iteration on 16 lanes)
__device__ int pair_inverse_iteration(C2<float> *W, int n, float sigma, unsigned char *sm, const PairHalf &H,
                                      C2<float> &z, float *lam, float *res)
{
    constexpr int LD = PLay::LD;
    C2<float> *col = reinterpret_cast<C2<float> *>(sm + PLay::ww);
    const int i = H.hl;
    if (i < n) W[i * LD + i].x -= sigma;
    __syncwarp(H.hm);
    if (!pair_chol<true>(W, n, col, H)) return -1;
    const float d = pair_strict_lower(W, n, H);
    const float tol = 1e-5f;
    float rprev = -1.f, cprev = 1.f, gap_good = 0.f;
    for (int it = 0; it < 10; ++it) {
        C2<float> x = z;
        pair_chol_solve(W, n, d, x, H);
        const float xx = hsum(cabs2(x), H.hm);
        const float xv = hsum(ccmul(x, z).x, H.hm);
        const float rho = sigma + xv / xx;
        const C2<float> r = cadd(z, cscale(x, sigma - rho));
        const float inv = rsqrtf(xx);
        const float rn = sqrtf(hsum(cabs2(r), H.hm)) * inv;
        z = cscale(x, inv);
        *lam = rho;
        *res = rn;
        if (rprev > 0.f) {
            const float c = rn / rprev;
            const float crate = max(c, cprev);
            if (crate < 0.9f) {
                const float gap = (rho - sigma) * (1.f / crate - 1.f);
                gap_good = gap;
                if (rn <= tol * gap) return 1;
            }
            if (it >= 3 && c > 0.9f) return (rn <= 20.f * tol * gap_good) ? 1 : 0;
            cprev = c;
        }
        rprev = rn;
    }
    return 0;
}

// |M|_F over the half's rows
__device__ __forceinline__ float pair_fro(const C2<float> *W, int n, const PairHalf &H)
{
    constexpr int LD = PLay::LD;
    float s = 0.f;
    if (H.hl < n)
        for (int j = 0; j < n; ++j) s += cabs2(W[H.hl * LD + j]);
    return sqrtf(hsum(s, H.hm));
}

// The MLE solve (evd semantics) of pixel pp by one half, the other half
// solving its own pixel at the same time.  Every lane of the warp calls it;
// go: this half has a pixel of this kind.  slab0: the warp's first slab (the
// Householder fall-back runs the whole warp on each half's slab).
__device__ void pair_mle(const KParams &P, long long pp, unsigned char *slab0, const PairRows &cp,
                         const PairHalf &H, bool go)
{
    constexpr int LD = PLay::LD;
    constexpr size_t SLAB = PLay::bytes_noc;
    unsigned char *sm = slab0 + H.h * SLAB;
    C2<float> *Wm = reinterpret_cast<C2<float> *>(sm + PLay::wm);
    const int hl = H.hl;
    const unsigned hm = H.hm;
    const int n = P.nb;
    const float thr = 1.0e-6f;
    const float amb = P.amb * float(n) * Eps<float>::v;

    // ---- record and coherence (evd.cpp:514-582) ----------------------------
    int npix = -1;
    if (go) npix = pair_load(P, pp, Wm, H);
    bool act = npix >= 0;
    __syncwarp();
    if (!__any_sync(0xffffffffu, act)) return;
    float cfro = 0.f;
    act = pair_coherence(P, pp, Wm, sm, cp, H, act, &cfro);
    if (act && npix < n) {
        // fewer SHPs than dates: Gamma is singular up to rounding (-2)
        put_code(P, pp, hl, -2);
        act = false;
    }

    // ---- lambda_min(C) vs 1e-6 (evd.cpp:600-619), shifts 1e-6 -+ the band
    {
        const float dC = amb * cfro;
        int r = 1;
        bool pend = act;
        for (int s = 0; s < 2; ++s) {
            if (!__any_sync(0xffffffffu, pend)) break;
            pair_copy_rows(cp, Wm, H, pend);
            if (pend) {
                const float sh = (s == 0) ? thr + dC : thr - dC;
                if (hl < n) Wm[hl * LD + hl].x -= sh;
                __syncwarp(hm);
                const bool ok = pair_chol<false>(Wm, n, reinterpret_cast<C2<float> *>(sm + PLay::vv), H);
                if (s == 0) {
                    if (ok) {
                        r = 1;
                        pend = false;
                    } else if (!(dC > 0.f)) {
                        r = -1;
                        pend = false;
                    }
                } else {
                    r = ok ? 0 : -1;
                    pend = false;
                }
            }
            __syncwarp();
        }
        if (act && r == 0) { defer_fp64(P, pp, hl); act = false; }
        if (act && r < 0) { put_code(P, pp, hl, -2); act = false; }
    }

    // ---- |C|, its inverse and M = inv|C| o C (evd.cpp:623-667) -------------
    const float lim = thr + amb * float(n);
    float xnorm = 0.f;
    {
        const int r = pair_build_M(cp, sm, Wm, H, act, n, P.cond_max, lim, amb, &xnorm);
        // not positive definite, so lambda_min(|C|) <= 0 < 1e-6 (evd.cpp:626-641)
        if (act && r < 0) put_code(P, pp, hl, -4);
        if (act && r == 0) defer_fp64(P, pp, hl);
        act = act && r > 0;
    }
    float tr = 0.f, dM = 0.f;
    bool dM_exact = false;
    if (act) {
        tr = hsum(hl < n ? Wm[hl * LD + hl].x : 0.f, hm) / float(n);
        dM = amb * sqrtf(float(n)) * xnorm;
    }
    C2<float> z = pair_power_start(cp, act ? n : 0, sm, H);

    // ---- smallest eigenpair by shifted inverse iteration (evd.cpp:670-686)
    int st = 0;
    float sig = 0.f, lam = 0.f, res = 0.f, rho1 = 0.f;
    bool run = false;
    if (act) {
        const C2<float> m = pair_matvec(Wm, n, reinterpret_cast<const C2<float> *>(sm + PLay::vv), H);
        const float rho0 = hsum(ccmul(z, m).x, hm);
        rho1 = min(rho0, 1.f);
        sig = P.shift * rho1;
        __syncwarp(hm);
        if (!(sig > thr + dM) && !dM_exact) { dM = amb * pair_fro(Wm, n, H); dM_exact = true; }
        run = sig > thr + dM;
        if (run) st = pair_inverse_iteration(Wm, n, sig, sm, H, z, &lam, &res);
    }
    // M again (the factorisation consumed it) for a second shift or for the
    // Householder path
    bool reb = run && st != 1;
    if (__any_sync(0xffffffffu, reb)) pair_build_M(cp, sm, Wm, H, reb, n, P.cond_max, lim, amb, &xnorm);
    if (reb) {
        if (hl == 0) atomicAdd(P.slow, 1);
        float sigma1;
        if (st == 0) {
            sigma1 = lam - 2.f * res;
            if (!(sigma1 > sig)) sigma1 = 0.f;
        } else {
            sigma1 = P.shift_backoff * rho1;
        }
        if (!(sigma1 > thr + dM) && !dM_exact) { dM = amb * pair_fro(Wm, n, H); dM_exact = true; }
        if (!(sigma1 > thr + dM)) {
            st = -1;
            reb = false;
        } else {
            sig = sigma1;
            st = pair_inverse_iteration(Wm, n, sig, sm, H, z, &lam, &res);
            reb = st != 1;
        }
    }
    if (__any_sync(0xffffffffu, reb)) pair_build_M(cp, sm, Wm, H, reb, n, P.cond_max, lim, amb, &xnorm);
    const bool hh_need = act && st != 1;
    float eig_hi = 0.f;
    if (hh_need) {
        eig_hi = tr * 1.0001f;
        if (!dM_exact) { dM = amb * pair_fro(Wm, n, H); dM_exact = true; }
    }
    // ---- Householder fall-back: the whole warp, one pixel at a time -------
    if (__any_sync(0xffffffffu, hh_need)) {
        const int lane = threadIdx.x & 31;
        for (int h = 0; h < 2; ++h) {
            if (!__shfl_sync(0xffffffffu, (int)hh_need, 16 * h)) continue;
            const int nh = __shfl_sync(0xffffffffu, n, 16 * h);
            const float hi = __shfl_sync(0xffffffffu, eig_hi, 16 * h);
            unsigned char *smh = slab0 + h * SLAB;
            C2<float> y0, y1;
            const float lh = warp_eigpair<float, PNP>(reinterpret_cast<C2<float> *>(smh + PLay::wm), nh, 1, -1e30f,
                                                      hi, smh, lane, y0, y1);
            C2<float> *vh = reinterpret_cast<C2<float> *>(smh + PLay::vv);
            __syncwarp();
            if (lane < nh) vh[lane] = y0;
            __syncwarp();
            if (H.h == h) {
                z = (hl < n) ? vh[hl] : cmk<float>(0.f, 0.f);
                lam = lh;
            }
            __syncwarp();
        }
    }
    if (hh_need) {
        if (lam < thr + dM && lam >= thr - dM) { defer_fp64(P, pp, hl); act = false; }
        else if (lam < thr) { put_code(P, pp, hl, -7); act = false; }
    }

    // ---- phases referenced to date mini-1 (evd.cpp:738-749) ---------------
    const long long plane = P.plane;
    float2 *phs = reinterpret_cast<float2 *>(sm + PLay::ph);
    const int mref = P.mini - 1;
    if (act) {
        const C2<float> zr = hbcast(z, mref, hm);
        const float zra2 = cabs2(zr);
        const C2<float> zru = (zra2 > 0.f) ? cscale(zr, rsqrtf(zra2)) : cmk<float>(1.f, 0.f);
        if (hl < n) {
            const float za2 = cabs2(z);
            const C2<float> u = (za2 > 0.f) ? cscale(z, rsqrtf(za2)) : cmk<float>(1.f, 0.f);
            const C2<float> pr = cmulc(u, zru);
            const float2 o = (hl == mref) ? make_float2(1.f, 0.f) : make_float2(pr.x, pr.y);
            phs[hl] = o;
            P.phase[hl * plane + pp] = o;
        }
        __syncwarp(hm);
        // compressed SLC (evd.cpp:752-762)
        float sr = 0.f, si = 0.f;
        if (hl < n && hl >= mref) {
            const float2 xs = __ldg(P.stack + hl * plane + pp);
            const float2 o = phs[hl];
            sr = __fadd_rn(__fmul_rn(xs.x, o.x), __fmul_rn(xs.y, o.y));
            si = __fsub_rn(__fmul_rn(xs.y, o.x), __fmul_rn(xs.x, o.y));
        }
        sr = hsum(sr, hm);
        si = hsum(si, hm);
        if (hl == 0) {
            const float den = float(n - mref);
            P.comp[pp] = make_float2(sr / den, si / den);
        }
    }

    // ---- temporal coherence (evd.cpp:768-786); every lane reads its row ----
    __syncwarp();
    const int ulim = (act && hl < n) ? n : 0;
    const float2 pi = (ulim > 0) ? phs[hl] : make_float2(0.f, 0.f);
    int cnt = max(ulim - hl - 1, 0);
    float wr = 0.f, wi = 0.f;
#pragma unroll 1
    for (int cc = 0; cc < PNP / 8; ++cc) {
        C2<float> cv[8];
        cp.load(0, cc, cv);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int j = 8 * cc + k;
            if (j <= hl || j >= ulim) continue;
            const C2<float> c = cv[k];
            const float ca2 = cabs2(c);
            const C2<float> u = (ca2 > 0.f) ? cscale(c, rsqrtf(ca2)) : cmk<float>(1.f, 0.f);
            const float2 pj = phs[j];
            const C2<float> v = cmul(u, cmk<float>(pj.x, pj.y));
            wr += v.x;
            wi += v.y;
        }
    }
    const C2<float> w = cmulc(cmk<float>(wr, wi), cmk<float>(pi.x, pi.y));
    const float sr = hsum(w.x, hm), si = hsum(w.y, hm);
    cnt = __reduce_add_sync(hm, cnt);
    if (act && hl == 0) {
        P.tcorr[pp] = sqrtf(sr * sr + si * si) / float(cnt);
        if (P.status) P.status[pp] = 0;
    }
}

}  // namespace
}  // namespace fpl
