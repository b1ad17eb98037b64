// pixel.cuh -- warp-per-pixel phase linking for sm_103a.
//
// One warp owns one pixel and runs the whole per-pixel body of the
// reference's evd / phase_link loop (src/evd/evd.cpp:514-786,
// src/phase_link/phase_link.cpp:480-665) out of registers and a per-warp
// shared-memory slab:
//   1. SHP gather: the window is walked 32 taps at a time; the nmap bits of a
//      tap chunk are compacted with a warp ballot and the selected samples
//      (all dates) are staged in shared memory;
//   2. Gamma = sum x x^H over the SHPs, register-blocked (each lane owns a
//      BR x 4 block of the upper triangle), then normalised to coherence;
//   3. eigen-solves in shared memory: power iteration for the EVD largest
//      eigenvector (Householder path when it converges slowly); for MLE a
//      Cholesky test of C, a symmetric-sweep inverse of |C|, then Householder
//      tridiagonalisation, warp multisection on the Sturm count, inverse
//      iteration on the tridiagonal and back-transformation;
//   4. phase referencing, compressed SLC and temporal coherence with warp
//      shuffles.
// T = float is the plain FP32 form.  Discrete decisions (eigenvalue < 1e-6,
// "is |Gamma| positive definite") whose FP32 answer lies inside a rounding
// band, and |Gamma| whose condition estimate is too large for an FP32
// inverse, are not settled in FP32: the pixel is appended to a list and
// recomputed by the same code instantiated with T = double.
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
    float amb;                          // width of the FP32 rounding band, in units of n*eps*|A|_F
    float cond_max;                     // largest inf-norm condition of |C| inverted in FP32
    float shift, shift_backoff;         // inverse-iteration shifts, in units of min(1, rho)
    int *fb_count;                      // FP64 work list (scratch): the 64-byte counter block of the
                                        // run: +0 list length, +16 err, +32 slow, +48 work cursor
    long long *fb_list;
    int fb_cap;
    unsigned *err;                      // error flags (scratch)
    int *slow;                          // pixels that left the fast eigen path (scratch)
    // mixed form: Gamma records from the tensor-core kernel
    float2 *cbuf;                       // [pixel - cbase][cstride floats] (pixel_load_gamma)
    int *cinfo;                         // [pixel - cbase]: SHP count, or CI_* below
    long long cbase;                    // first pixel of the buffers
    int cstride;                        // floats per record
};

enum { CI_CENTRE = -1, CI_FEW = -2, CI_DEFER = -3 };

// one launch's share of a batched launch: the Gamma kernel's segment
// (tiles [tile_offset, next segment's tile_offset)) and the solve and FP64
// kernels' entry (pixels [px_offset, next entry's px_offset))
struct BoxSeg {
    KParams P;
    long long tile_offset;
};
struct BatchEntry {
    KParams P;
    long long px_offset;   // first pixel of this entry in the class's concatenated range
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
// acc += a * b, acc -= a * b
template <typename T> __device__ __forceinline__ void cfma(C2<T> &acc, C2<T> a, C2<T> b)
{
    acc.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
    acc.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
}

// b -= a * y and b -= conj(a) * y as fused multiply-adds
template <typename T> __device__ __forceinline__ void fms_mul(C2<T> &b, C2<T> a, C2<T> y)
{
    b.x = fma(-a.x, y.x, fma(a.y, y.y, b.x));
    b.y = fma(-a.x, y.y, fma(-a.y, y.x, b.y));
}
template <typename T> __device__ __forceinline__ void fms_cmul(C2<T> &b, C2<T> a, C2<T> y)
{
    b.x = fma(-a.x, y.x, fma(-a.y, y.y, b.x));
    b.y = fma(-a.x, y.y, fma(a.y, y.x, b.y));
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

// fast division where only a rounding-level result is needed (Sturm counts)
__device__ __forceinline__ float fdiv_fast(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double fdiv_fast(double a, double b) { return a / b; }
__device__ __forceinline__ float rsqrt_t(float a) { return rsqrtf(a); }
__device__ __forceinline__ double rsqrt_t(double a) { return rsqrt(a); }

// ------------------------------------------------------------------------
// per-warp shared-memory slab layout
// ------------------------------------------------------------------------
__host__ __device__ constexpr size_t align16(size_t x) { return (x + 15) & ~size_t(15); }
__host__ __device__ constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }

template <typename T, int NP> struct Lay {
    static constexpr int LD = NP + 1;        // matrix row stride (odd: conflict-free columns)
    static constexpr int XS = NP + 2;        // staging row stride in float2 (16-byte rows)
    static constexpr size_t mat = sizeof(C2<T>) * NP * LD;
    static constexpr size_t wm = 0;                                   // work: staging / Cholesky / M / tridiag
    static constexpr size_t wm_bytes = align16(cmax(mat, sizeof(float2) * 32 * XS));
    static constexpr size_t xr = wm + align16(mat / 2);               // real sweep matrix: upper half of wm
    static constexpr size_t vv = wm + wm_bytes;                       // complex vector v
    static constexpr size_t ww = align16(vv + sizeof(C2<T>) * NP);    // complex vector w
    static constexpr size_t tu = align16(ww + sizeof(C2<T>) * NP);    // tau
    static constexpr size_t dd = align16(tu + sizeof(C2<T>) * NP);    // d
    static constexpr size_t ee = align16(dd + sizeof(T) * NP);        // e
    static constexpr size_t e2 = align16(ee + sizeof(T) * NP);        // e^2
    static constexpr size_t yy = align16(e2 + sizeof(T) * NP);        // y / row k / 1/sqrt(P)
    static constexpr size_t wk = align16(yy + sizeof(T) * NP);        // 5*NP scratch (lane 0)
    static constexpr size_t ph = align16(wk + sizeof(T) * 5 * NP);    // phases (float2)
    // the coherence C comes last: kernels that keep C in tensor memory
    // allocate only bytes_noc per warp
    static constexpr size_t bytes_noc = align16(ph + sizeof(float2) * NP);
    static constexpr size_t cm = bytes_noc;                           // coherence C
    static constexpr size_t bytes = cm + align16(mat);
};

// FP64 at 64 dates keeps C in tensor memory during the eigen-solve (see
// CInTmem), so the coherence needs shared memory only while Gamma is summed
// and normalised: it sits right after the gather staging, over the work
// matrix (which the solve uses only after C has been copied out), and the
// vectors follow it.  91.6 KB per warp instead of 141 KB: two warps per SM.
template <> struct Lay<double, 64> {
    static constexpr int NP = 64;
    static constexpr int LD = NP + 1;
    static constexpr int XS = NP + 2;
    static constexpr size_t mat = sizeof(C2<double>) * NP * LD;
    static constexpr size_t wm = 0;
    static constexpr size_t stage = align16(sizeof(float2) * 32 * XS);  // gather staging at wm
    static constexpr size_t wm_bytes = align16(cmax(mat, stage));
    static constexpr size_t xr = wm + align16(mat / 2);
    static constexpr size_t cm = stage;                               // Gamma / C while it is formed
    static constexpr size_t vv = cmax(wm + wm_bytes, cm + align16(mat));
    static constexpr size_t ww = align16(vv + sizeof(C2<double>) * NP);
    static constexpr size_t tu = align16(ww + sizeof(C2<double>) * NP);
    static constexpr size_t dd = align16(tu + sizeof(C2<double>) * NP);
    static constexpr size_t ee = align16(dd + sizeof(double) * NP);
    static constexpr size_t e2 = align16(ee + sizeof(double) * NP);
    static constexpr size_t yy = align16(e2 + sizeof(double) * NP);
    static constexpr size_t wk = align16(yy + sizeof(double) * NP);
    static constexpr size_t ph = align16(wk + sizeof(double) * 5 * NP);
    static constexpr size_t bytes_noc = align16(ph + sizeof(float2) * NP);
    static constexpr size_t bytes = bytes_noc;
};

// while Gamma is summed the gather staging, the coherence and the vectors
// (1/sqrt(P) among them) are all live, so they must not overlap; the work
// matrix may overlap the coherence (it is used only after C moved out)
static_assert(Lay<double, 64>::cm >= Lay<double, 64>::wm + Lay<double, 64>::stage, "staging overlaps C");
static_assert(Lay<double, 64>::vv >= Lay<double, 64>::cm + Lay<double, 64>::mat, "vectors overlap C");
static_assert(Lay<double, 64>::vv >= Lay<double, 64>::wm + Lay<double, 64>::wm_bytes, "vectors overlap W");
static_assert(2 * Lay<double, 64>::bytes <= 224 * 1024, "two warps per CTA");

// kernels whose warps hold C in tensor memory in the FP64 form
template <typename T, int NP> struct CInTmem {
    static constexpr bool value = sizeof(T) == 8 && NP == 64;
};

// The plain FP32 form at <= 32 dates keeps C in tensor memory as well (rows
// as CRowsTmem, as the mixed form's solve does), which halves the slab and
// raises the warps per SM: Gamma is accumulated in registers in one pass,
// so C is formed over the gather staging (no longer read by then) and moved
// to tensor memory before the solve reuses that memory.
template <typename T, int NP> struct CRowsTmemF {
    static constexpr bool value = sizeof(T) == 4 && NP <= 32;
};
// where the pixel kernels form C in the slab
template <typename T, int NP> struct CmOffset {
    static constexpr size_t value = CRowsTmemF<T, NP>::value ? Lay<T, NP>::wm : Lay<T, NP>::cm;
};
// tensor-memory columns of a CTA whose warps hold np-date coherence rows
// (CRowsTmem<np>, four warps per lane quadrant): a power of two >= 32
__device__ __forceinline__ int tmem_cols_for(int warps, int np)
{
    int need = ((warps + 3) / 4) * 2 * np * ((np + 31) / 32), cols = 32;
    while (cols < need) cols <<= 1;
    return cols;
}
// shared memory per warp of the pixel kernels (k_pixels, k_batch)
template <typename T, int NP> struct KPixWarp {
    static constexpr size_t bytes = CRowsTmemF<T, NP>::value ? Lay<T, NP>::bytes_noc : Lay<T, NP>::bytes;
};

// ------------------------------------------------------------------------
// Access to the rows of the coherence C.  Lane l owns rows l and l + 32;
// rows are read and written in chunks of 8 complex entries (columns 8c ..
// 8c+7).  Every lane of the warp calls load / store together (the tensor-
// memory form requires it); rows >= NP read as zero.
// ------------------------------------------------------------------------
template <typename T, int NP> struct CRowsSmem {
    C2<T> *C;
    int lane;
    __device__ __forceinline__ void load(int h, int c, C2<T> (&v)[8]) const
    {
        const int i = lane + 32 * h;
        const C2<T> *r = C + i * (NP + 1) + 8 * c;
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = (i < NP) ? r[k] : cmk<T>(T(0), T(0));
    }
    __device__ __forceinline__ void store(int h, int c, const C2<T> (&v)[8]) const
    {
        const int i = lane + 32 * h;
        if (i >= NP) return;
        C2<T> *r = C + i * (NP + 1) + 8 * c;
#pragma unroll
        for (int k = 0; k < 8; ++k) r[k] = v[k];
    }
    __device__ __forceinline__ void fence() const { __syncwarp(); }
};

// C in tensor memory (FP32, NP <= 64): the warp owns 2*NP 32-bit columns
// of its 32 TMEM lanes per row slot; lane l holds row l (and row l + 32 in a
// second block of 2*NP columns when NP = 64), Re and Im interleaved.  The solver
// kernels issue no MMA: tensor memory is extra per-warp storage there,
// which frees shared memory for more resident warps.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
        "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16};"
        :: "r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
           "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
        : "memory");
}

template <int NP> struct CRowsTmem {
    static_assert(NP <= 64, "at most two rows per lane");
    // row slot h of the lane (row lane + 32 h) starts 2*NP columns after slot h-1
    static constexpr uint32_t kColsPerWarp = 2u * NP * ((NP + 31) / 32);
    uint32_t taddr;      // lane quadrant << 16 | first column of the warp
    __device__ __forceinline__ void load(int h, int c, C2<float> (&v)[8]) const
    {
        uint32_t r[16];
        tmem_ld16(taddr + (uint32_t)(2 * NP * h) + 16u * (uint32_t)c, r);
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = cmk<float>(__uint_as_float(r[2 * k]), __uint_as_float(r[2 * k + 1]));
    }
    __device__ __forceinline__ void store(int h, int c, const C2<float> (&v)[8]) const
    {
        uint32_t r[16];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            r[2 * k] = __float_as_uint(v[k].x);
            r[2 * k + 1] = __float_as_uint(v[k].y);
        }
        tmem_st16(taddr + (uint32_t)(2 * NP * h) + 16u * (uint32_t)c, r);
    }
    __device__ __forceinline__ void fence() const
    {
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
};

// The same rows of an FP64 C: a complex double is four 32-bit columns, so
// row slot h starts 4*NP columns after slot h-1 (at 64 dates the warp's
// two row slots fill the 512 columns of its lane quadrant).
template <int NP> struct CRowsTmemD {
    static_assert(NP <= 64, "at most two rows per lane");
    static constexpr uint32_t kColsPerWarp = 4u * NP * ((NP + 31) / 32);
    uint32_t taddr;      // lane quadrant << 16 | first column of the warp
    __device__ __forceinline__ void load(int h, int c, C2<double> (&v)[8]) const
    {
        const uint32_t a = taddr + (uint32_t)(4 * NP * h) + 32u * (uint32_t)c;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            uint32_t r[16];
            tmem_ld16(a + 16u * (uint32_t)half, r);
#pragma unroll
            for (int k = 0; k < 4; ++k)
                v[4 * half + k] = cmk<double>(__hiloint2double((int)r[4 * k + 1], (int)r[4 * k]),
                                              __hiloint2double((int)r[4 * k + 3], (int)r[4 * k + 2]));
        }
    }
    __device__ __forceinline__ void store(int h, int c, const C2<double> (&v)[8]) const
    {
        const uint32_t a = taddr + (uint32_t)(4 * NP * h) + 32u * (uint32_t)c;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            uint32_t r[16];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const C2<double> x = v[4 * half + k];
                r[4 * k] = (uint32_t)__double2loint(x.x);
                r[4 * k + 1] = (uint32_t)__double2hiint(x.x);
                r[4 * k + 2] = (uint32_t)__double2loint(x.y);
                r[4 * k + 3] = (uint32_t)__double2hiint(x.y);
            }
            tmem_st16(a + 16u * (uint32_t)half, r);
        }
    }
    __device__ __forceinline__ void fence() const
    {
        asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    }
};

// tensor memory of a CTA: warp 0 allocates `cols` columns (a power of two
// >= 32) and gives up the right to allocate more; every thread gets the base
// address.  Call from every thread; tmem_free_cta releases them.
__device__ __forceinline__ uint32_t tmem_alloc_cta(uint32_t *slot, int warp, uint32_t cols)
{
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"((uint32_t)__cvta_generic_to_shared(slot)), "r"(cols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    return *slot;
}
__device__ __forceinline__ void tmem_free_cta(uint32_t tbase, int warp, uint32_t cols)
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tbase), "r"(cols) : "memory");
}

// number of row slots (h) and 8-entry chunks (c) per lane
template <int NP> struct RowShape {
    static constexpr int H = (NP + 31) / 32;
    static constexpr int CH = NP / 8;
};

// y = C x through a row policy (lane-distributed x in smem xv, y in y0 / y1)
template <typename T, int NP, typename CP>
__device__ void rows_matvec(const CP &cp, int n, const C2<T> *xv, C2<T> &y0, C2<T> &y1, int lane)
{
#pragma unroll
    for (int h = 0; h < RowShape<NP>::H; ++h) {
        C2<T> a = cmk<T>(T(0), T(0));
#pragma unroll 1
        for (int c = 0; c < RowShape<NP>::CH; ++c) {
            C2<T> v[8];
            cp.load(h, c, v);
#pragma unroll
            for (int k = 0; k < 8; k += 2) {
                const int j = 8 * c + k;
                C2<T> x0, x1;
                if (sizeof(T) == 4) {
                    const float4 q = *reinterpret_cast<const float4 *>(xv + j);
                    x0 = cmk<T>(T(q.x), T(q.y));
                    x1 = cmk<T>(T(q.z), T(q.w));
                } else {
                    x0 = xv[j];
                    x1 = xv[j + 1];
                }
                if (j < n) cfma(a, v[k], x0);
                if (j + 1 < n) cfma(a, v[k + 1], x1);
            }
        }
        const int i = lane + 32 * h;
        if (i >= n) a = cmk<T>(T(0), T(0));
        if (h == 0) y0 = a; else y1 = a;
    }
    if (RowShape<NP>::H == 1) y1 = cmk<T>(T(0), T(0));
}

// ------------------------------------------------------------------------
// warp Cholesky (lower, in place) of the complex Hermitian matrix in A:
// returns false at the first pivot that is not > 0 (or NaN), like zpotrf's
// test (AJJ <= 0 .or. disnan(AJJ)).  col: NP complex smem scratch.
// STORE: keep L in the lower triangle with 1 / L_jj on the diagonal (for the
// triangular solves); otherwise only the Schur complements are updated.
// ------------------------------------------------------------------------
template <typename T, int LD, int NP, bool STORE = false>
__device__ bool warp_chol_c(C2<T> *A, int n, C2<T> *col, int lane)
{
    for (int j = 0; j < n; ++j) {
        const T piv = A[j * LD + j].x;
        if (!(piv > T(0))) return false;
        const T r = rsqrt_t(piv);
        // scaled column j (l_k, k > j) into col[] for broadcast reads; zeros elsewhere
        for (int k = lane; k < NP; k += 32) {
            C2<T> l = (k > j && k < n) ? cscale(A[k * LD + j], r) : cmk<T>(T(0), T(0));
            col[k] = l;
            if (STORE && k > j && k < n) A[k * LD + j] = l;
        }
        if (STORE && lane == 0) A[j * LD + j] = cmk<T>(r, T(0));
        __syncwarp();
        for (int i = j + 1 + lane; i < n; i += 32) {
            const C2<T> li = col[i];
            C2<T> *__restrict__ Ai = A + i * LD;
            // A[i][k] -= l_i conj(l_k), k in (j, i]; col[k] = 0 for k <= j.
            // Four columns per step, loads issued before the stores.
            for (int k = (j + 1) & ~3; k <= i; k += 4) {
                C2<T> l[4], a[4];
                if (sizeof(T) == 4) {
                    const float4 v0 = *reinterpret_cast<const float4 *>(col + k);
                    const float4 v1 = *reinterpret_cast<const float4 *>(col + k + 2);
                    l[0] = cmk<T>(T(v0.x), T(v0.y)); l[1] = cmk<T>(T(v0.z), T(v0.w));
                    l[2] = cmk<T>(T(v1.x), T(v1.y)); l[3] = cmk<T>(T(v1.z), T(v1.w));
                } else {
#pragma unroll
                    for (int u = 0; u < 4; ++u) l[u] = col[k + u];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) a[u] = Ai[k + u];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    a[u].x -= li.x * l[u].x + li.y * l[u].y;
                    a[u].y -= li.y * l[u].x - li.x * l[u].y;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (k + u > j && k + u <= i) Ai[k + u] = a[u];
            }
        }
        __syncwarp();
    }
    return true;
}

// Two elimination steps per pass (FP32, NP <= 32, row i on lane i): the
// scaled columns j and j+1 are published together and every row below
// takes both rank-1 updates in one pass over its entries, as fused
// multiply-adds.  Same pivot tests and STORE layout as warp_chol_c.  Entries
// right of the diagonal are left with intermediate values (only the lower
// triangle and the diagonal are read afterwards).  col: 2 x NP complex.
template <int LD, int NP, bool STORE = false>
__device__ bool warp_chol_c2(C2<float> *A, int n, C2<float> *col, int lane)
{
    static_assert(NP <= 32, "one row per lane");
    C2<float> *cA = col, *cB = col + NP;
    const int i = lane;
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
            // pivot j+1 after the step-j update: a_(j+1)(j+1) - |l_(j+1)|^2
            const C2<float> ln = cmk<float>(__shfl_sync(0xffffffffu, l1.x, j + 1), __shfl_sync(0xffffffffu, l1.y, j + 1));
            const float p2 = fmaf(-ln.y, ln.y, fmaf(-ln.x, ln.x, A[(j + 1) * LD + j + 1].x));
            if (!(p2 > 0.f)) return false;
            r2 = rsqrtf(p2);
            if (b2) {
                C2<float> a = Ai[j + 1];                    // a - l_i conj(l_(j+1))
                a.x = fmaf(-l1.x, ln.x, fmaf(-l1.y, ln.y, a.x));
                a.y = fmaf(-l1.y, ln.x, fmaf(l1.x, ln.y, a.y));
                l2 = cmk<float>(a.x * r2, a.y * r2);
            }
        }
        if (i < NP) {
            cA[i] = l1;
            cB[i] = l2;
        }
        if (STORE) {
            if (i == j) Ai[j] = cmk<float>(r1, 0.f);
            else if (b1) Ai[j] = l1;
            if (two) {
                if (i == j + 1) Ai[j + 1] = cmk<float>(r2, 0.f);
                else if (b2) Ai[j + 1] = l2;
            }
        }
        __syncwarp();
        if (b2) {
            // a_ik -= l1_i conj(l1_k) + l2_i conj(l2_k), k in (j+1, i]
            // two entries per step (j is even, so k0 starts at j + 2)
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
        __syncwarp();
    }
    return true;
}

// The Cholesky factorisation used by the solvers: the two-step form for
// FP32 with one row per lane, else warp_chol_c.  col: 2 x NP complex.
template <typename T, int LD, int NP, bool STORE = false>
__device__ __forceinline__ bool warp_chol_any(C2<T> *A, int n, C2<T> *col, int lane)
{
    if constexpr (sizeof(T) == 4 && NP <= 32)
        return warp_chol_c2<LD, NP, STORE>(A, n, col, lane);
    else
        return warp_chol_c<T, LD, NP, STORE>(A, n, col, lane);
}

// Turns the factor of warp_chol_c<STORE> (L below the diagonal, 1/L_jj on
// it, anything above it) into the strict-lower form of warp_chol_solve:
// zeros on and above the diagonal, 1/L_ii returned per lane (d0: row lane,
// d1: row lane + 32).
template <typename T, int LD, int NP>
__device__ void chol_strict_lower(C2<T> *L, int n, T &d0, T &d1, int lane)
{
#pragma unroll
    for (int h = 0; h < (NP + 31) / 32; ++h) {
        const int i = lane + 32 * h;
        T d = T(0);
        if (i < n) {
            C2<T> *Li = L + i * LD;
            d = Li[i].x;
            for (int k = i; k < n; ++k) Li[k] = cmk<T>(T(0), T(0));
        }
        if (h == 0) d0 = d;
        else d1 = d;
    }
    __syncwarp();
}

// Solves (L L^H) x = b for a factor in strict-lower form (see
// chol_strict_lower).  b / x are lane-distributed (element i on lane i%32,
// slot i/32).  Because L_ij = 0 for j >= i, every lane takes every update
// unpredicated: step j broadcasts b_j / L_jj from lane j (final after step
// j-1) and each row subtracts its multiple, so a step is two multiplies,
// two shuffles, one shared load and four fused multiply-adds.  Rows at or
// beyond n come back zero.
template <typename T, int LD, int NP>
__device__ void warp_chol_solve(const C2<T> *L, int n, T d0, T d1, C2<T> &b0, C2<T> &b1, int lane)
{
    const C2<T> *L0 = L + lane * LD;
    const C2<T> *L1 = L + (lane + 32) * LD;
    // forward: L y = b
#pragma unroll 2
    for (int j = 0; j < n; ++j) {
        C2<T> s = (NP <= 32 || j < 32) ? cscale(b0, d0) : cscale(b1, d1);
        C2<T> y;
        y.x = __shfl_sync(0xffffffffu, s.x, j & 31);
        y.y = __shfl_sync(0xffffffffu, s.y, j & 31);
        fms_mul(b0, L0[j], y);
        if (NP > 32) fms_mul(b1, L1[j], y);
    }
    b0 = cscale(b0, d0);
    if (NP > 32) b1 = cscale(b1, d1);
    // backward: L^H x = y, b_i -= conj(L_ji) x_j
#pragma unroll 2
    for (int j = n - 1; j >= 0; --j) {
        C2<T> s = (NP <= 32 || j < 32) ? cscale(b0, d0) : cscale(b1, d1);
        C2<T> x;
        x.x = __shfl_sync(0xffffffffu, s.x, j & 31);
        x.y = __shfl_sync(0xffffffffu, s.y, j & 31);
        fms_cmul(b0, L[j * LD + lane], x);
        if (NP > 32) fms_cmul(b1, L[j * LD + lane + 32], x);
    }
    b0 = (lane < n) ? cscale(b0, d0) : cmk<T>(T(0), T(0));
    if (NP > 32) b1 = (lane + 32 < n) ? cscale(b1, d1) : cmk<T>(T(0), T(0));
}

// lambda_min(A) vs thr for a complex Hermitian A (lower triangle read):
// +1 certainly above, -1 certainly at or below, 0 inside [thr-delta, thr+delta].
template <typename T, int LD, int NP, typename CP>
__device__ int lam_min_test_c(const CP &cp, C2<T> *W, C2<T> *col, int n, T thr, T delta, int lane)
{
    const int nsh = delta > T(0) ? 2 : 1;
    for (int s = 0; s < nsh; ++s) {
        T sh = (nsh == 1) ? thr : (s == 0 ? thr + delta : thr - delta);
        __syncwarp();
#pragma unroll
        for (int h = 0; h < RowShape<NP>::H; ++h) {
            const int i = lane + 32 * h;
#pragma unroll 1
            for (int c = 0; c < RowShape<NP>::CH; ++c) {
                C2<T> v[8];
                cp.load(h, c, v);
                if (i < NP) {
#pragma unroll
                    for (int k = 0; k < 8; ++k) W[i * LD + 8 * c + k] = v[k];
                }
            }
        }
        __syncwarp();
        for (int i = lane; i < n; i += 32) W[i * LD + i].x -= sh;
        __syncwarp();
        bool ok = warp_chol_any<T, LD, NP>(W, n, col, lane);
        __syncwarp();
        if (nsh == 1) return ok ? 1 : -1;
        if (s == 0 && ok) return 1;
        if (s == 1 && !ok) return -1;
    }
    return 0;
}

// ------------------------------------------------------------------------
// symmetric sweep (Gauss-Jordan) inverse of a real symmetric matrix, in
// place: sweeping every index leaves -inv(A).  The sweep pivots are the
// LDL^T pivots, so "a pivot <= 0" is the same decision as a failing
// Cholesky factorisation.  Lane i owns row i; all lanes work every step.
// rowk: NP real smem scratch.  On success A holds inv(A) and *inf_norm the
// largest absolute row sum of the inverse.
// ------------------------------------------------------------------------
template <typename T, int LD, int NP>
__device__ bool warp_sweep_inverse(T *A, int n, T *rowk, T *inf_norm, int lane, int *kfail = nullptr)
{
    for (int k = 0; k < n; ++k) {
        for (int j = lane; j < NP; j += 32) rowk[j] = (j < n) ? A[k * LD + j] : T(0);
        __syncwarp();
        const T p = rowk[k];
        if (!(p > T(0))) {
            if (kfail) *kfail = k;           // rowk holds row k (see abs_not_pd)
            return false;
        }
        const T rp = T(1) / p;
        for (int i = lane; i < n; i += 32) {
            T *__restrict__ Ai = A + i * LD;
            // row k: a_kj / p;  other rows: a_ij - (a_ik / p) a_kj
            const bool own = (i == k);
            const T f = rowk[i] * rp;
            const T a = own ? T(0) : T(1);
            const T b = own ? rp : -f;
            int j = 0;
            for (; j + 8 <= n; j += 8) {
                T r[8], x[8];
                if (sizeof(T) == 4) {
                    const float4 v0 = *reinterpret_cast<const float4 *>(rowk + j);
                    const float4 v1 = *reinterpret_cast<const float4 *>(rowk + j + 4);
                    r[0] = T(v0.x); r[1] = T(v0.y); r[2] = T(v0.z); r[3] = T(v0.w);
                    r[4] = T(v1.x); r[5] = T(v1.y); r[6] = T(v1.z); r[7] = T(v1.w);
                } else {
#pragma unroll
                    for (int u = 0; u < 8; ++u) r[u] = rowk[j + u];
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) x[u] = Ai[j + u];
#pragma unroll
                for (int u = 0; u < 8; ++u) Ai[j + u] = fma(b, r[u], a * x[u]);
            }
            for (; j < n; ++j) Ai[j] = fma(b, rowk[j], a * Ai[j]);
            Ai[k] = own ? -rp : f;
        }
        __syncwarp();
    }
    T mx = T(0);
    for (int i = lane; i < n; i += 32) {
        T s = T(0);
        for (int j = 0; j < n; ++j) {
            T v = -A[i * LD + j];
            A[i * LD + j] = v;
            s += abs(v);
        }
        mx = max(mx, s);
    }
    *inf_norm = warp_max(mx);
    __syncwarp();
    return true;
}

// The same sweep for FP32 and NP <= 32 with each lane's row in registers:
// at step k lane k publishes its row (which is also column k) to a shared
// buffer and every lane updates its own row from it, so the matrix is read
// from shared memory once and written back once instead of at every step.
// Same sweep as warp_sweep_inverse; the pivot row's update is written
// x + (1/p - 1) x.  The loop over k is not unrolled (its body is the same
// for every k), which keeps the code small.  rowb: 2 x NP + 2 floats of
// shared memory (16-byte aligned): two row buffers and two pivot slots.
template <int LD, int NP>
__device__ bool warp_sweep_inverse_rows(float *A, int n, float *rowb, float *inf_norm, int lane,
                                        int *kfail = nullptr)
{
    static_assert(NP <= 32 && NP % 8 == 0, "one row per lane");
    float x[NP];
#pragma unroll
    for (int j = 0; j < NP; ++j) x[j] = (lane < n && j < n) ? A[lane * LD + j] : 0.f;
    // Lane k publishes row k with its k-th entry replaced by p - 1 (p, the
    // pivot a_kk, is kept beside the row): x + (-f)(p - 1) turns a_ik into
    // a_ik / p = f in the same fused multiply-add as the rest of the row,
    // so column k needs no register chosen by k.  Lane k's own entry
    // becomes 2 - 1/p instead of -1/p; no later step reads a row's
    // diagonal after that row was swept, and the 2 is taken off at the end.
#pragma unroll 1
    for (int k = 0; k < n; ++k) {
        float *rk = rowb + (k & 1) * NP;
        float *pk = rowb + 2 * NP + (k & 1);
        if (lane == k) {
#pragma unroll
            for (int j = 0; j < NP; j += 4) *reinterpret_cast<float4 *>(rk + j) = make_float4(x[j], x[j + 1], x[j + 2], x[j + 3]);
            const float v = rk[k];
            *pk = v;
            rk[k] = v - 1.f;
        }
        __syncwarp();
        const float p = *pk;
        if (!(p > 0.f)) {
            if (kfail) *kfail = k;           // rk holds row k, entries j < k (see abs_not_pd)
            return false;
        }
        const float rp = 1.f / p;
        const bool own = (lane == k);
        // row k: a_kj / p;  other rows: a_ij - (a_ik / p) a_kj  (a_ik = a_ki)
        const float f = ((lane < NP) ? rk[lane] : 0.f) * rp;
        const float bm = own ? rp - 1.f : -f;
#pragma unroll
        for (int j = 0; j < NP; j += 4) {
            const float4 r = *reinterpret_cast<const float4 *>(rk + j);
            x[j] = fmaf(bm, r.x, x[j]);
            x[j + 1] = fmaf(bm, r.y, x[j + 1]);
            x[j + 2] = fmaf(bm, r.z, x[j + 2]);
            x[j + 3] = fmaf(bm, r.w, x[j + 3]);
        }
    }
    __syncwarp();
    float s = 0.f;
    if (lane < n) {
#pragma unroll
        for (int j = 0; j < NP; ++j) {
            if (j < n) {
                const float v = (j == lane) ? 2.f - x[j] : -x[j];
                A[lane * LD + j] = v;
                s += fabsf(v);
            }
        }
    }
    *inf_norm = warp_max(s);
    __syncwarp();
    return true;
}

// ------------------------------------------------------------------------
// Householder tridiagonalisation (restates the zhetd2/zlarfg reduction):
// Q^H A Q = T, Q = H(0)..H(n-2), reflector v_k in A[k+1.., k] (v_k[0] = 1),
// tau_k in tau, d / e real.  A is full Hermitian storage, row i on lane i%32.
// vv / ww: NP complex smem vectors (broadcast copies of v and w).
// ------------------------------------------------------------------------
template <typename T, int LD, int NP>
__device__ void warp_tridiag(C2<T> *A, int n, T *d, T *e, C2<T> *tau, C2<T> *vv, C2<T> *ww, int lane)
{
    for (int k = 0; k < n - 1; ++k) {
        T s = T(0);
        for (int i = k + 2 + lane; i < n; i += 32) s += cabs2(A[i * LD + k]);
        s = warp_sum(s);
        const C2<T> alpha = A[(k + 1) * LD + k];
        C2<T> t = cmk<T>(T(0), T(0));
        C2<T> scal = cmk<T>(T(1), T(0));
        T beta;
        if (s == T(0) && alpha.y == T(0)) {
            beta = alpha.x;
        } else {
            T nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + s);
            beta = alpha.x >= T(0) ? -nrm : nrm;
            t = cmk<T>((beta - alpha.x) / beta, -alpha.y / beta);
            scal = cdiv(cmk<T>(T(1), T(0)), cmk<T>(alpha.x - beta, alpha.y));
        }
        const bool act = (t.x != T(0) || t.y != T(0));
        __syncwarp();
        // v: zeros up to k, 1 at k+1, scaled column below; kept in column k of A
        for (int i = lane; i < NP; i += 32) {
            C2<T> v = cmk<T>(T(0), T(0));
            if (i == k + 1) v = cmk<T>(T(1), T(0));
            else if (i > k + 1 && i < n) v = act ? cmul(A[i * LD + k], scal) : A[i * LD + k];
            if (i > k && i < n) A[i * LD + k] = v;
            vv[i] = v;
        }
        if (lane == 0) {
            tau[k] = t;
            e[k] = beta;
            d[k] = A[k * LD + k].x;
        }
        __syncwarp();
        if (act) {
            // p = t * A22 v ; K = -1/2 t (p^H v) ; w = p + K v
            const int j0 = (k + 1) & ~1;
            C2<T> pv = cmk<T>(T(0), T(0));
            C2<T> p[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int i = lane + 32 * h;
                p[h] = cmk<T>(T(0), T(0));
                if (h * 32 >= NP) continue;
                if (i > k && i < n) {
                    const C2<T> *Ai = A + i * LD;
                    C2<T> acc0 = cmk<T>(T(0), T(0)), acc1 = cmk<T>(T(0), T(0));
                    for (int j = j0; j < n; j += 2) {
                        C2<T> v0, v1;
                        if (sizeof(T) == 4) {
                            float4 q = *reinterpret_cast<const float4 *>(vv + j);
                            v0 = cmk<T>(T(q.x), T(q.y));
                            v1 = cmk<T>(T(q.z), T(q.w));
                        } else {
                            v0 = vv[j];
                            v1 = vv[j + 1];
                        }
                        cfma(acc0, Ai[j], v0);
                        if (j + 1 < n) cfma(acc1, Ai[j + 1], v1);
                    }
                    p[h] = cmul(t, cadd(acc0, acc1));
                    pv = cadd(pv, ccmul(p[h], vv[i]));
                }
            }
            pv.x = warp_sum(pv.x);
            pv.y = warp_sum(pv.y);
            const C2<T> K = cscale(cmul(t, pv), T(-0.5));
            for (int i = lane; i < NP; i += 32) {
                C2<T> w = cmk<T>(T(0), T(0));
                if (i > k && i < n) w = cadd(p[i >= 32 ? 1 : 0], cmul(K, vv[i]));
                ww[i] = w;
            }
            __syncwarp();
            // A22 -= v w^H + w v^H (vv / ww are zero at indices <= k)
            for (int i = k + 1 + lane; i < n; i += 32) {
                C2<T> *Ai = A + i * LD;
                const C2<T> vi = vv[i], wi = ww[i];
                for (int j = j0; j < n; j += 2) {
                    C2<T> v0, v1, w0, w1;
                    if (sizeof(T) == 4) {
                        float4 q = *reinterpret_cast<const float4 *>(vv + j);
                        float4 r = *reinterpret_cast<const float4 *>(ww + j);
                        v0 = cmk<T>(T(q.x), T(q.y));
                        v1 = cmk<T>(T(q.z), T(q.w));
                        w0 = cmk<T>(T(r.x), T(r.y));
                        w1 = cmk<T>(T(r.z), T(r.w));
                    } else {
                        v0 = vv[j]; v1 = vv[j + 1]; w0 = ww[j]; w1 = ww[j + 1];
                    }
                    if (j > k) Ai[j] = csub(Ai[j], cadd(cmulc(vi, w0), cmulc(wi, v0)));
                    if (j + 1 < n) Ai[j + 1] = csub(Ai[j + 1], cadd(cmulc(vi, w1), cmulc(wi, v1)));
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
        q = (d[i] - sigma) - fdiv_fast(e2[i - 1], q);
        if (abs(q) <= pivmin) q = -pivmin;
        cnt += q < T(0);
    }
    return cnt;
}

// index-th (1-based ascending) eigenvalue of the tridiagonal (d, e) by
// 33-way warp multisection.  [lo_hint, hi_hint] narrows the Gershgorin
// interval when the caller knows a bound.
template <typename T>
__device__ T warp_tridiag_eig(const T *d, const T *e, T *e2, int n, int index, T lo_hint, T hi_hint,
                              T *tnorm_out, int lane)
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
    const T pivmin = Eps<T>::tiny * max(T(1), em) * T(4);
    const T tnorm = max(abs(gl), abs(gu));
    const T fudge = T(2.1) * eps * tnorm * T(n) + T(2) * pivmin;
    T lo = max(gl - fudge, lo_hint), hi = min(gu + fudge, hi_hint);
    if (!(lo < hi)) { lo = gl - fudge; hi = gu + fudge; }
    for (int it = 0; it < 64; ++it) {
        const T tol = T(2) * eps * max(abs(lo), abs(hi)) + pivmin;
        if (hi - lo <= tol) break;
        const T w = (hi - lo) / T(33);
        T sig = lo + w * T(lane + 1);
        if (lane == 31) sig = min(sig, hi);
        const int c = sturm(d, e2, n, sig, pivmin);
        const unsigned ge = __ballot_sync(0xffffffffu, c >= index);
        const int f = ge ? (__ffs(ge) - 1) : 32;        // first point with count >= index
        const T s_f = __shfl_sync(0xffffffffu, sig, f & 31);
        const T s_p = __shfl_sync(0xffffffffu, sig, (f - 1) & 31);
        const T nlo = (f == 0) ? lo : s_p;
        const T nhi = (f == 32) ? hi : s_f;
        if (!(nhi < hi || nlo > lo)) break;            // no progress (rounding floor)
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
        T *rdg = wk, *u1 = wk + n, *u2 = wk + 2 * n, *l = wk + 3 * n, *pv = wk + 4 * n;
        const T eps = Eps<T>::v * (tnorm > T(0) ? tnorm : T(1));
        T dgi = d[0] - lam;
        T u1i = (n > 1) ? e[0] : T(0);
        T dnext = (n > 1) ? d[1] - lam : T(0);
        T u1next = (n > 2) ? e[1] : T(0);
        for (int i = 0; i < n - 1; ++i) {
            const T sub = e[i];
            T rd, ul1, ul2 = T(0), li, piv = T(0);
            if (abs(dgi) >= abs(sub)) {
                if (dgi == T(0)) dgi = eps;
                rd = T(1) / dgi;
                li = sub * rd;
                ul1 = u1i;
                dnext -= li * u1i;          // next row keeps u1next
            } else {
                const T mult = dgi / sub;
                rd = T(1) / sub;
                ul1 = dnext;
                ul2 = u1next;
                const T nd = u1i - mult * dnext;
                u1next = -mult * u1next;
                dnext = nd;
                li = mult;
                piv = T(1);
            }
            rdg[i] = rd; u1[i] = ul1; u2[i] = ul2; l[i] = li; pv[i] = piv;
            dgi = dnext;
            u1i = u1next;
            dnext = (i + 2 < n) ? d[i + 2] - lam : T(0);
            u1next = (i + 3 < n) ? e[i + 2] : T(0);
        }
        if (dgi == T(0)) dgi = eps;
        rdg[n - 1] = T(1) / dgi;
        u1[n - 1] = T(0); u2[n - 1] = T(0);
        for (int i = 0; i < n; ++i) y[i] = T(1);
        for (int it = 0; it < 2; ++it) {
            for (int i = 0; i < n - 1; ++i) {
                if (pv[i] != T(0)) { T t = y[i]; y[i] = y[i + 1]; y[i + 1] = t - l[i] * y[i]; }
                else y[i + 1] -= l[i] * y[i];
            }
            T y1 = T(0), y2 = T(0), mx = T(0);
            for (int i = n - 1; i >= 0; --i) {
                T t = (y[i] - u1[i] * y1 - u2[i] * y2) * rdg[i];
                y[i] = t;
                y2 = y1;
                y1 = t;
                mx = max(mx, abs(t));
            }
            if (!(mx > T(0)) || !isfinite(mx)) { for (int i = 0; i < n; ++i) y[i] = T(1); continue; }
            const T r = T(1) / mx;
            for (int i = 0; i < n; ++i) y[i] *= r;
        }
    }
    __syncwarp();
}

// Eigenpair of the Hermitian matrix in W (destroyed): index-th eigenvalue
// (1-based ascending).  Returns the eigenvalue; lane i gets z_i (and z_{i+32}).
template <typename T, int NP>
__device__ T warp_eigpair(C2<T> *W, int n, int index, T lo_hint, T hi_hint, unsigned char *sm,
                          int lane, C2<T> &z0, C2<T> &z1)
{
    using L = Lay<T, NP>;
    constexpr int LD = L::LD;
    T *d = reinterpret_cast<T *>(sm + L::dd);
    T *e = reinterpret_cast<T *>(sm + L::ee);
    T *e2 = reinterpret_cast<T *>(sm + L::e2);
    T *y = reinterpret_cast<T *>(sm + L::yy);
    T *wk = reinterpret_cast<T *>(sm + L::wk);
    C2<T> *tau = reinterpret_cast<C2<T> *>(sm + L::tu);
    C2<T> *vv = reinterpret_cast<C2<T> *>(sm + L::vv);
    C2<T> *ww = reinterpret_cast<C2<T> *>(sm + L::ww);
    if (n == 1) {
        z0 = cmk<T>(T(1), T(0));
        z1 = cmk<T>(T(0), T(0));
        return W[0].x;
    }
    warp_tridiag<T, LD, NP>(W, n, d, e, tau, vv, ww, lane);
    T tnorm;
    const T lam = warp_tridiag_eig<T>(d, e, e2, n, index, lo_hint, hi_hint, &tnorm, lane);
    tridiag_inverse_iteration<T>(d, e, n, lam, tnorm, y, wk, lane);
    const int i0 = lane, i1 = lane + 32;
    z0 = (i0 < n) ? cmk<T>(y[i0], T(0)) : cmk<T>(T(0), T(0));
    z1 = (i1 < n) ? cmk<T>(y[i1], T(0)) : cmk<T>(T(0), T(0));
    for (int k = n - 2; k >= 0; --k) {
        const C2<T> t = tau[k];
        if (t.x == T(0) && t.y == T(0)) continue;
        C2<T> s = cmk<T>(T(0), T(0));
        if (i0 >= k + 1 && i0 < n) s = cadd(s, ccmul(W[i0 * LD + k], z0));
        if (NP > 32 && i1 >= k + 1 && i1 < n) s = cadd(s, ccmul(W[i1 * LD + k], z1));
        s.x = warp_sum(s.x);
        s.y = warp_sum(s.y);
        s = cmul(t, s);
        if (i0 >= k + 1 && i0 < n) z0 = csub(z0, cmul(s, W[i0 * LD + k]));
        if (NP > 32 && i1 >= k + 1 && i1 < n) z1 = csub(z1, cmul(s, W[i1 * LD + k]));
    }
    return lam;
}

// Largest eigenvector of the Hermitian C by power iteration.  Returns true
// with z (lane-distributed) when the residual test passes; false when the
// iteration converges too slowly (the caller then uses the Householder path).
template <typename T, int NP, typename CP>
__device__ bool warp_power(const CP &cp, int n, unsigned char *sm, int lane, C2<T> &z0, C2<T> &z1,
                           T *lam_out)
{
    using L = Lay<T, NP>;
    C2<T> *vv = reinterpret_cast<C2<T> *>(sm + L::vv);
    const int i0 = lane, i1 = lane + 32;
    // start: row sums (C * 1)
    for (int i = lane; i < NP; i += 32) vv[i] = cmk<T>(i < n ? T(1) : T(0), T(0));
    __syncwarp();
    T rprev = T(-1);
    const T tol = (sizeof(T) == 4) ? T(4e-6) : T(1e-13);
    for (int it = 0; it < 96; ++it) {
        C2<T> u[2];
        rows_matvec<T, NP>(cp, n, vv, u[0], u[1], lane);
        // rho = v^H u (v normalised after the first pass), residual u - rho v
        const C2<T> v0 = (i0 < n) ? vv[i0] : cmk<T>(T(0), T(0));
        const C2<T> v1 = (NP > 32 && i1 < n) ? vv[i1] : cmk<T>(T(0), T(0));
        T vn = warp_sum(cabs2(v0) + cabs2(v1));
        T rho = warp_sum(ccmul(v0, u[0]).x + ccmul(v1, u[1]).x) / vn;
        const C2<T> r0 = csub(u[0], cscale(v0, rho)), r1 = csub(u[1], cscale(v1, rho));
        const T rn = sqrt(warp_sum(cabs2(r0) + cabs2(r1)) / vn);
        const T un = warp_sum(cabs2(u[0]) + cabs2(u[1]));
        const T inv = rsqrt_t(un);
        __syncwarp();
        if (i0 < n) vv[i0] = cscale(u[0], inv);
        if (NP > 32 && i1 < n) vv[i1] = cscale(u[1], inv);
        __syncwarp();
        // eigenvector error ~ rn / gap; the contraction rn/rprev estimates
        // lambda2/lambda1, so the gap is about rho (1 - ratio)
        const T ratio = (rprev > T(0)) ? min(rn / rprev, T(1)) : T(1);
        rprev = rn;
        if (it >= 2 && rn <= tol * rho * max(T(1) - ratio, T(0.05))) {
            z0 = (i0 < n) ? vv[i0] : cmk<T>(T(0), T(0));
            z1 = (NP > 32 && i1 < n) ? vv[i1] : cmk<T>(T(0), T(0));
            *lam_out = rho;
            return true;
        }
        if (it >= 8 && ratio > T(0.8)) return false;   // slow: use the Householder path
    }
    return false;
}

// y = A x for the Hermitian A in smem (lane-distributed x / y)
template <typename T, int LD, int NP>
__device__ void warp_matvec(const C2<T> *A, int n, const C2<T> *xv, C2<T> &y0, C2<T> &y1, int lane)
{
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int i = lane + 32 * h;
        C2<T> u = cmk<T>(T(0), T(0));
        if (h * 32 < NP && i < n) {
            const C2<T> *Ai = A + i * LD;
            C2<T> a0 = cmk<T>(T(0), T(0)), a1 = cmk<T>(T(0), T(0));
#pragma unroll 2
            for (int j = 0; j < n; j += 2) {
                C2<T> v0, v1;
                if (sizeof(T) == 4) {
                    const float4 q = *reinterpret_cast<const float4 *>(xv + j);
                    v0 = cmk<T>(T(q.x), T(q.y));
                    v1 = cmk<T>(T(q.z), T(q.w));
                } else {
                    v0 = xv[j];
                    v1 = xv[j + 1];
                }
                cfma(a0, Ai[j], v0);
                if (j + 1 < n) cfma(a1, Ai[j + 1], v1);
            }
            u = cadd(a0, a1);
        }
        if (h == 0) y0 = u; else y1 = u;
    }
}

// A few power iterations on C from the all-ones vector: a start vector for
// the MLE inverse iteration (the EVD and MLE solutions are close).  Leaves
// the normalised vector lane-distributed in z0 / z1 and in vv.
template <typename T, int NP, typename CP>
__device__ void warp_power_start(const CP &cp, int n, int iters, unsigned char *sm, int lane,
                                 C2<T> &z0, C2<T> &z1)
{
    using L = Lay<T, NP>;
    C2<T> *vv = reinterpret_cast<C2<T> *>(sm + L::vv);
    for (int i = lane; i < NP; i += 32) vv[i] = cmk<T>(i < n ? T(1) : T(0), T(0));
    __syncwarp();
    for (int it = 0; it < iters; ++it) {
        C2<T> u0, u1;
        rows_matvec<T, NP>(cp, n, vv, u0, u1, lane);
        const T inv = rsqrt_t(warp_sum(cabs2(u0) + cabs2(u1)));
        z0 = cscale(u0, inv);
        z1 = cscale(u1, inv);
        __syncwarp();
        if (lane < n) vv[lane] = z0;
        if (NP > 32 && lane + 32 < n) vv[lane + 32] = z1;
        __syncwarp();
    }
}

// Smallest eigenpair of the Hermitian M (in W, destroyed) by inverse
// iteration with the shift sigma.  A successful Cholesky factorisation of
// M - sigma I certifies sigma < lambda_1, so the iteration converges to the
// smallest eigenpair; its rate is (lambda_1 - sigma) / (lambda_2 - sigma).
// The start vector comes in z0 / z1.  Returns 1 when converged (z = unit
// eigenvector, *lam = Rayleigh quotient), 0 when converging too slowly
// (z, *lam, *res = the current iterate, Rayleigh quotient and residual), -1
// when M - sigma I is not positive definite.
template <typename T, int NP>
__device__ int warp_inverse_iteration(C2<T> *W, int n, T sigma, unsigned char *sm, int lane,
                                      C2<T> &z0, C2<T> &z1, T *lam, T *res)
{
    using L = Lay<T, NP>;
    constexpr int LD = L::LD;
    C2<T> *col = reinterpret_cast<C2<T> *>(sm + L::ww);
    for (int i = lane; i < n; i += 32) W[i * LD + i].x -= sigma;
    __syncwarp();
    if (!warp_chol_any<T, LD, NP, true>(W, n, col, lane)) return -1;
    T d0 = T(0), d1 = T(0);
    chol_strict_lower<T, LD, NP>(W, n, d0, d1, lane);
    const T tol = (sizeof(T) == 4) ? T(1e-5) : T(1e-12);
    T rprev = T(-1), cprev = T(1), gap_good = T(0);
    for (int it = 0; it < 10; ++it) {
        C2<T> x0 = z0, x1 = z1;
        warp_chol_solve<T, LD, NP>(W, n, d0, d1, x0, x1, lane);
        const T xx = warp_sum(cabs2(x0) + cabs2(x1));
        const T xv = warp_sum(ccmul(x0, z0).x + ccmul(x1, z1).x);
        const T rho = sigma + xv / xx;
        // M x - rho x = z + (sigma - rho) x
        const C2<T> r0 = cadd(z0, cscale(x0, sigma - rho)), r1 = cadd(z1, cscale(x1, sigma - rho));
        const T inv = rsqrt_t(xx);
        const T rn = sqrt(warp_sum(cabs2(r0) + cabs2(r1))) * inv;
        z0 = cscale(x0, inv);
        z1 = cscale(x1, inv);
        *lam = rho;
        *res = rn;
        if (rprev > T(0)) {
            // eigenvector error ~ rn / (lambda_2 - lambda_1).  The residual
            // contracts by (lambda_1 - sigma)/(lambda_2 - sigma) per step, so
            // the gap is about (rho - sigma)(1/c - 1); the larger of the last
            // two contractions is used (early steps contract faster).
            const T c = rn / rprev;
            const T crate = max(c, cprev);
            if (crate < T(0.9)) {
                const T gap = (rho - sigma) * (T(1) / crate - T(1));
                gap_good = gap;
                if (rn <= tol * gap) return 1;
            }
            // residual no longer decreasing: rounding floor
            if (it >= 3 && c > T(0.9)) return (rn <= T(20) * tol * gap_good) ? 1 : 0;
            cprev = c;
        }
        rprev = rn;
    }
    return 0;
}

// power steps that refine the vector of the not-positive-definite proof
constexpr int kNotPdSteps = 2;

// |C| not positive definite, proved from a failed sweep of |C|.  When the
// sweep meets the pivot p <= 0 at step k, the entries w_j (j < k) of row k
// solve |C|_SS w = |C|_Sk over the swept indices S, and v = (-w, 1, 0, ..)
// has v^T |C| v = p in exact arithmetic.  The form is evaluated again from
// the coherence rows (|C| formed as the sweep formed it): a value below
// -(g s + band |v|^2), with s = |v|^T |C| |v| and g its evaluation's
// rounding bound, and band the bound on the spectral difference from the
// reference's |C| that the other decisions use, proves that the reference's
// |C| has a negative eigenvalue (any vector serves as the witness).  When v
// falls short, up to kNotPdSteps power steps on ||C||_inf I - |C| move it
// toward the eigenvector of the smallest eigenvalue and the test is taken
// again.  rk: row k (entries j < k are read); amb: the band per unit of
// ||C||_F, whose sum is taken in the first pass; ub: NP entries of scratch.
// Every lane calls it.
template <typename T, int NP, typename CP>
__device__ bool abs_not_pd(const CP &cp, const T *rk, int k, int n, T amb, T *ub, int lane)
{
    constexpr bool fp32 = sizeof(T) == 4;
    constexpr int H = RowShape<NP>::H;
    for (int i = lane; i < NP; i += 32) ub[i] = (i < k) ? -rk[i] : (i == k ? T(1) : T(0));
    __syncwarp();
    const T g = T(2 * (n + 1)) * Eps<T>::v;
    T band = T(0), anorm = T(0);
    for (int it = 0;; ++it) {
        T q = T(0), s = T(0), v2 = T(0), f2 = T(0), rmax = T(0);
        T u[H];
#pragma unroll
        for (int h = 0; h < H; ++h) {
            const int i = lane + 32 * h;
            const T vi = (i < n) ? ub[i] : T(0);
            T yq = T(0), ys = T(0), rs = T(0);
#pragma unroll 1
            for (int c = 0; c < RowShape<NP>::CH; ++c) {
                C2<T> cv[8];
                cp.load(h, c, cv);
#pragma unroll
                for (int kk = 0; kk < 8; ++kk) {
                    const int j = 8 * c + kk;
                    if (i >= n || j >= n) continue;
                    const T m2 = cabs2(cv[kk]);
                    f2 += m2;
                    const T a = (i == j) ? T(1) : (fp32 ? m2 * rsqrt_t(max(m2, T(1e-37))) : sqrt(m2));
                    const T vj = ub[j];
                    yq = fma(a, vj, yq);
                    ys = fma(a, abs(vj), ys);
                    rs += a;
                }
            }
            q = fma(vi, yq, q);
            s = fma(abs(vi), ys, s);
            v2 = fma(vi, vi, v2);
            rmax = max(rmax, rs);
            u[h] = (i < n) ? yq : T(0);
        }
        q = warp_sum(q);
        s = warp_sum(s);
        v2 = warp_sum(v2);
        if (it == 0) {
            band = amb * sqrt(warp_sum(f2));
            anorm = warp_max(rmax);
        }
        if (q < -(g * s + band * v2)) return true;
        if (it == kNotPdSteps) return false;
        // v <- ||C||_inf v - |C| v, scaled by its largest entry
        T um = T(0);
#pragma unroll
        for (int h = 0; h < H; ++h) {
            const int i = lane + 32 * h;
            u[h] = (i < n) ? fma(anorm, ub[i], -u[h]) : T(0);
            um = max(um, abs(u[h]));
        }
        um = warp_max(um);
        if (!(um > T(0))) return false;
        const T ru = T(1) / um;
        __syncwarp();
#pragma unroll
        for (int h = 0; h < H; ++h) {
            const int i = lane + 32 * h;
            if (i < n) ub[i] = u[h] * ru;
        }
        __syncwarp();
    }
}

// ------------------------------------------------------------------------
// per-pixel driver
// ------------------------------------------------------------------------
// power iterations on C from the all-ones vector that start the MLE
// inverse iteration (one: a second cost more solve time than the inverse
// iteration steps it saved)
constexpr int kPowerStartIters = 1;

// register block of the upper triangle of Gamma each lane accumulates
// (BR rows x BC columns): 8 x 4 in FP32 and 4 x 4 in FP64 give 20 and 36
// blocks at 32 dates; at 16 dates FP32 uses 4 x 2 blocks, so that 20 lanes
// share the sums instead of the 6 that 8 x 4 blocks would leave busy
template <typename T, int NP> struct BlockShape {
    static constexpr int BR = sizeof(T) == 4 ? (NP <= 16 ? 4 : 8) : 4;
    static constexpr int BC = (sizeof(T) == 4 && NP <= 16) ? 2 : 4;
};

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

// next entry of the FP64 work list for this warp: warps draw entries from a
// cursor in the run's counter block (zeroed with it), so the SMs whose
// pixels were cheap take more of them
__device__ __forceinline__ long long fb_next(const KParams &P, int lane)
{
    int q = 0;
    if (lane == 0) q = atomicAdd(P.fb_count + 12, 1);
    return __shfl_sync(0xffffffffu, q, 0);
}

__device__ __forceinline__ void defer_fp64(const KParams &P, long long pp, int lane)
{
    if (lane == 0) {
        int idx = atomicAdd(P.fb_count, 1);
        if (idx < P.fb_cap) P.fb_list[idx] = pp;
        else atomicOr(P.err, ERR_FB_OVERFLOW);
    }
}

__device__ __forceinline__ void put_code(const KParams &P, long long pp, int lane, int code)
{
    if (lane == 0) {
        P.tcorr[pp] = float(code);
        if (P.status) P.status[pp] = code;
    }
}

// Gather, Gamma and coherence (evd.cpp:514-582).  Returns the SHP count
// with C in the warp's slab, or -1 when the pixel is finished (skipped or
// coded) and its outputs are written.
// Gamma (upper triangle and diagonal of the warp's C slab) to coherence
// (evd.cpp:569-582, phase_link.cpp:527-538): C_ij = Gamma_ij / sqrt(P_i P_j),
// lower triangle by conjugation, unit diagonal.  A non-finite result is
// reported as the failure of the first eigen call; returns false then.
template <typename T, int NP>
__device__ bool gamma_to_coherence(const KParams &P, long long pp, C2<T> *Cm, unsigned char *sm, int lane)
{
    using L = Lay<T, NP>;
    constexpr int LD = L::LD;
    T *yv = reinterpret_cast<T *>(sm + L::yy);
    const int n = P.nb;
    const bool plink = (P.semantics == SEM_PL);
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
        put_code(P, pp, lane, (!plink && P.method != M_MLE) ? -6 : -1);
        return false;
    }
    return true;
}

template <typename T, int NP>
__device__ int pixel_coherence(const KParams &P, long long pp, unsigned char *sm, int lane)
{
    using L = Lay<T, NP>;
    constexpr int LD = L::LD;
    constexpr int XS = L::XS;
    constexpr int BR = BlockShape<T, NP>::BR, BC = BlockShape<T, NP>::BC;
    constexpr int NBR = NP / BR, NBC = NP / BC;
    constexpr int CPR = BR / BC;   // first block column of block row R is CPR*R
    constexpr int NBLK = NBR * NBC - CPR * NBR * (NBR - 1) / 2;
    constexpr int PASSES = (NBLK + 31) / 32;

    static_assert(!CRowsTmemF<T, NP>::value || PASSES == 1, "C over the staging needs Gamma in registers");
    C2<T> *Cm = reinterpret_cast<C2<T> *>(sm + CmOffset<T, NP>::value);
    C2<T> *Wm = reinterpret_cast<C2<T> *>(sm + L::wm);
    float2 *Xs = reinterpret_cast<float2 *>(sm + L::wm);
    T *Xr = reinterpret_cast<T *>(sm + L::xr);
    T *yv = reinterpret_cast<T *>(sm + L::yy);
    C2<T> *col = reinterpret_cast<C2<T> *>(sm + L::vv);
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
        return -1;
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
            for (int t = 0; t < n; ++t) {
                dst[t] = __ldg(src);
                src += plane;
            }
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
        return -1;
    }

    if (!gamma_to_coherence<T, NP>(P, pp, Cm, sm, lane)) return -1;
    return npix;
}


// Eigen-solve and outputs for a pixel whose coherence C is reached through
// the row policy cp (the warp's slab, or tensor memory), evd.cpp:584-786,
// phase_link.cpp:540-665.
template <typename T, int NP, typename CP>
__device__ void pixel_solve(const KParams &P, long long pp, unsigned char *sm, int lane, int npix,
                            const CP &cp, T cfro = T(-1))
{
    using L = Lay<T, NP>;
    using RS = RowShape<NP>;
    constexpr int LD = L::LD;
    C2<T> *Wm = reinterpret_cast<C2<T> *>(sm + L::wm);
    T *Xr = reinterpret_cast<T *>(sm + L::xr);
    T *yv = reinterpret_cast<T *>(sm + L::yy);
    C2<T> *col = reinterpret_cast<C2<T> *>(sm + L::vv);
    float2 *phs = reinterpret_cast<float2 *>(sm + L::ph);
    const int n = P.nb;
    const long long plane = P.plane;
    const bool plink = (P.semantics == SEM_PL);

    const bool fp32 = sizeof(T) == 4;
    const T amb = T(P.amb) * T(n) * Eps<T>::v;          // rounding band unit (FP32 only)
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
    auto fro_c = [&]() {
        T s = T(0);
#pragma unroll
        for (int h = 0; h < RS::H; ++h) {
            const int i = lane + 32 * h;
#pragma unroll 1
            for (int c = 0; c < RS::CH; ++c) {
                C2<T> v[8];
                cp.load(h, c, v);
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (i < nn && 8 * c + k < nn) s += cabs2(v[k]);
            }
        }
        return sqrt(warp_sum(s));
    };
    // |C| into Xr (unit diagonal), then its sweep inverse.  Returns
    // +1 inverted (X = inv|C| in Xr), -1 not positive definite, 0 undecided
    // in FP32 (rounding band or condition too large).
    T xnorm = T(0);     // inf-norm of inv|C| from the last abs_inverse()
    auto abs_inverse = [&]() -> int {
        T rs = T(0);
#pragma unroll
        for (int h = 0; h < RS::H; ++h) {
            const int i = lane + 32 * h;
            T s = T(0);
#pragma unroll 1
            for (int c = 0; c < RS::CH; ++c) {
                C2<T> v[8];
                cp.load(h, c, v);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int j = 8 * c + k;
                    const T m2 = cabs2(v[k]);
                    const T a = (i == j) ? T(1) : (fp32 ? m2 * rsqrt_t(max(m2, T(1e-37))) : sqrt(m2));
                    if (i < nn && j < nn) {
                        Xr[i * LD + j] = a;
                        s += a;
                    }
                }
            }
            rs = max(rs, s);
        }
        const T anorm = warp_max(rs);          // |C| inf-norm
        __syncwarp();
        bool ok;
        int kfail = 0;
        const T *rk;
        if constexpr (sizeof(T) == 4 && NP <= 32) {
            float *rowb = reinterpret_cast<float *>(sm + L::wk);
            ok = warp_sweep_inverse_rows<LD, NP>(reinterpret_cast<float *>(Xr), nn, rowb, &xnorm, lane, &kfail);
            rk = reinterpret_cast<const T *>(rowb + (kfail & 1) * NP);
        } else {
            ok = warp_sweep_inverse<T, LD, NP>(Xr, nn, yv, &xnorm, lane, &kfail);
            rk = yv;
        }
        if (!fp32) return ok ? 1 : -1;
        if (!ok) {
            // FP32 pivot failure: |C| clearly not positive definite, or
            // positive definite but too close to singular for FP32 (settled
            // in FP64)
            T *ub = reinterpret_cast<T *>(sm + L::wk) + 3 * NP;     // past the sweep's rows
            return abs_not_pd<T, NP>(cp, rk, kfail, nn, amb, ub, lane) ? -1 : 0;
        }
        if (!(anorm * xnorm <= T(P.cond_max))) return 0;
        return 1;
    };

    const bool mle_evd = !plink && P.method == M_MLE;
    if (mle_evd) {
        // evd.cpp:598-686
        if (npix < n) {
            // fewer SHPs than dates: Gamma has rank <= npix < n, so its
            // smallest eigenvalue is 0 up to FP32 product rounding (far
            // below 1e-6): the reference reports -2.
            put_code(P, pp, lane, -2);
            return;
        }
        const T dC = fp32 ? amb * (cfro >= T(0) ? cfro : fro_c()) : T(0);
        const int r = lam_min_test_c<T, LD, NP>(cp, Wm, col, n, thr, dC, lane);
        if (r == 0) { defer_fp64(P, pp, lane); return; }
        if (r < 0) { put_code(P, pp, lane, -2); return; }
    }
    if (mle_evd || plink) {
        // |C| and its inverse: evd.cpp:623-664 (check, then inverse);
        // phase_link.cpp:540-618 (MLE if |C| is invertible, else EVD).  One
        // call site for both modules.
        const int r = abs_inverse();
        if (r == 0) { defer_fp64(P, pp, lane); return; }
        if (plink) {
            if (r > 0) {
                mode = 0;
            } else {
                mode = 1;
                pstatus = 3;
            }
        } else {
            if (r < 0) {
                // not positive definite (FP64, or proved in FP32 by
                // abs_not_pd), so lambda_min(|C|) <= 0 < 1e-6
                put_code(P, pp, lane, -4);
                return;
            }
            if (!fp32) {
                // lambda_min(|C|) >= 1/||inv|C|||_inf settles the 1e-6 test
                // unless the inverse is large
                T xn = T(0);
                for (int i = lane; i < n; i += 32) {
                    T s = T(0);
                    for (int j = 0; j < n; ++j) s += abs(Xr[i * LD + j]);
                    xn = max(xn, s);
                }
                xn = warp_max(xn);
                if (!(xn < T(1) / thr)) {
                    // decide with the Cholesky test of |C| - 1e-6 I (this work
                    // matrix overlaps the inverse, which is then recomputed)
                    __syncwarp();
#pragma unroll
                    for (int h = 0; h < RS::H; ++h) {
                        const int i = lane + 32 * h;
#pragma unroll 1
                        for (int c = 0; c < RS::CH; ++c) {
                            C2<T> v[8];
                            cp.load(h, c, v);
#pragma unroll
                            for (int k = 0; k < 8; ++k) {
                                const int j = 8 * c + k;
                                if (i < n && j <= i)
                                    Wm[i * LD + j] = cmk<T>((i == j) ? T(1) - thr : sqrt(cabs2(v[k])), T(0));
                            }
                        }
                    }
                    __syncwarp();
                    if (!warp_chol_c<T, LD, NP>(Wm, n, col, lane)) {
                        put_code(P, pp, lane, -4);
                        return;
                    }
                    __syncwarp();
                    abs_inverse();
                }
            } else {
                // lambda_min(|C|) >= 1 / ||inv|C|||_inf, so a small inverse
                // norm settles the 1e-6 test; anything else is settled in FP64
                const T dA = amb * T(n);
                if (!(T(1) / xnorm > thr + dA)) { defer_fp64(P, pp, lane); return; }
            }
            mode = 0;
        }
    } else {
        if (P.method == M_STBAS) {                       // evd.cpp:695-706
#pragma unroll
            for (int h = 0; h < RS::H; ++h) {
                const int i = lane + 32 * h;
#pragma unroll 1
                for (int c = 0; c < RS::CH; ++c) {
                    C2<T> v[8];
                    cp.load(h, c, v);
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const int j = 8 * c + k;
                        if (j - i > P.bw || i - j > P.bw) v[k] = cmk<T>(T(0), T(0));
                    }
                    cp.store(h, c, v);
                }
            }
            cp.fence();
        }
        mode = 1;
    }

    // ---- the eigenvector --------------------------------------------------
    C2<T> z0, z1;
    T lam = T(0), eig_lo = T(0), eig_hi = T(0), dM = T(0);
    int eig_index = 0;   // > 0: eigenpair of Wm by this index on the Householder path
    if (mode == 0) {
        // M = inv(|C|) o C (evd.cpp:667); Xr shares bytes with Wm, so each
        // lane reads its inverse row into registers before M is written.
        auto form_M = [&]() {
#pragma unroll
            for (int h = 0; h < RS::H; ++h) {
                const int i = lane + 32 * h;
                T xrow[NP];
#pragma unroll
                for (int j = 0; j < NP; ++j) xrow[j] = (i < nn && j < nn) ? Xr[i * LD + j] : T(0);
                __syncwarp();
#pragma unroll
                for (int c = 0; c < RS::CH; ++c) {
                    C2<T> v[8];
                    cp.load(h, c, v);
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const int j = 8 * c + k;
                        if (i < nn && j < nn) Wm[i * LD + j] = cscale(v[k], xrow[j]);
                    }
                }
                __syncwarp();
            }
        };
        form_M();
        // smallest eigenpair (evd.cpp:670-686).  M = inv|C| o C is positive
        // semi-definite (Schur product), and its smallest eigenvalue is at
        // most the mean of its diagonal.
        T tr = T(0);
        for (int i = lane; i < n; i += 32) tr += Wm[i * LD + i].x;
        tr = warp_sum(tr) / T(n);
        // rounding band of the decisions on M's eigenvalues, amb |M|_F.  The
        // common path needs only sigma > 1e-6 + band, which the bound
        // |M|_F <= sqrt(n) |inv|C||_inf (|M_ij| <= |inv|C|_ij|, and the
        // 2-norm of the symmetric inv|C| is at most its inf-norm) settles
        // without a pass over M; the exact value is formed while M is in Wm
        // whenever a decision is not settled by the bound.
        const bool need_band = fp32 && !plink;
        dM = need_band ? amb * sqrt(T(n)) * xnorm : T(0);
        bool dM_exact = !need_band;
        auto exact_dM = [&]() {
            if (!dM_exact) {
                dM = amb * fro(Wm);
                dM_exact = true;
            }
        };
        __syncwarp();
        bool done = false;
        if (fp32) {
            // inverse iteration from the EVD direction, shifted just below
            // the Rayleigh quotient (the smallest eigenvalue is close to 1)
            warp_power_start<T, NP>(cp, n, kPowerStartIters, sm, lane, z0, z1);
            C2<T> *vv = reinterpret_cast<C2<T> *>(sm + L::vv);
            C2<T> m0, m1;
            warp_matvec<T, LD, NP>(Wm, n, vv, m0, m1, lane);
            const T rho0 = warp_sum(ccmul(z0, m0).x + ccmul(z1, m1).x);
            // P.shift (0.1%) below the Rayleigh quotient (or 1); if M - sigma I
            // is not positive definite the shift was above lambda_1 and a
            // second attempt backs off to P.shift_backoff (3%) below
            const T rho1 = min(rho0, T(1));
            const T sigma = T(P.shift) * rho1;
            __syncwarp();
            if (!(sigma > thr + dM)) exact_dM();               // M is still in Wm
            if (sigma > thr + dM) {
                // one call site for the iteration and for rebuilding M (the
                // factorisation consumes it), so each is inlined once
                T sig = sigma;
                int st = 0;
                for (int attempt = 0; attempt < 2; ++attempt) {
                    T lam, res;
                    st = warp_inverse_iteration<T, NP>(Wm, n, sig, sm, lane, z0, z1, &lam, &res);
                    if (st != 1) {
                        // M for a second shift or for the Householder path
                        __syncwarp();
                        abs_inverse();
                        form_M();
                    }
                    if (st == 1 || attempt == 1) break;
                    if (lane == 0) atomicAdd(P.slow, 1);
                    T sigma1;
                    if (st == 0) {
                        // slow: shift again just below the current Rayleigh
                        // quotient (lambda_1 >= rho - res when the iterate is
                        // closest to v_1; the Cholesky test verifies the shift)
                        sigma1 = lam - T(2) * res;
                        if (!(sigma1 > sig)) sigma1 = T(0);
                    } else {
                        sigma1 = T(P.shift_backoff) * rho1;
                    }
                    if (!(sigma1 > thr + dM)) exact_dM();       // M was rebuilt in Wm
                    if (!(sigma1 > thr + dM)) {
                        st = -1;
                        break;
                    }
                    sig = sigma1;
                }
                // converged: lambda_1 > sigma > 1e-6 + band, the -7 test passes
                done = (st == 1);
            }
        }
        if (!done) {
            eig_index = 1;
            eig_lo = T(-1e30);
            eig_hi = tr * T(1.0001);
            exact_dM();            // M is in Wm (rebuilt after a failed attempt)
        }
    } else {
        bool ok = warp_power<T, NP>(cp, n, sm, lane, z0, z1, &lam);
        if (!ok) {
            if (lane == 0 && fp32) atomicAdd(P.slow, 1);
#pragma unroll
            for (int h = 0; h < RS::H; ++h) {
                const int i = lane + 32 * h;
#pragma unroll 1
                for (int c = 0; c < RS::CH; ++c) {
                    C2<T> v[8];
                    cp.load(h, c, v);
#pragma unroll
                    for (int k = 0; k < 8; ++k)
                        if (i < n && 8 * c + k < n) Wm[i * LD + 8 * c + k] = v[k];
                }
            }
            __syncwarp();
            eig_index = n;
            eig_lo = T(0.999);
            eig_hi = T(1e30);
        }
    }
    // Householder path, one call site for both methods
    if (eig_index) lam = warp_eigpair<T, NP>(Wm, n, eig_index, eig_lo, eig_hi, sm, lane, z0, z1);
    if (mode == 0) {
        if (eig_index && !plink) {
            if (fp32 && lam < thr + dM && lam >= thr - dM) { defer_fp64(P, pp, lane); return; }
            if (lam < thr) { put_code(P, pp, lane, -7); return; }
        }
    } else {
        // trace(C) = n, so lambda_max >= 1: the -7 test of evd.cpp:718-726
        // cannot trigger for a finite C.
        if (!plink && lam < thr) { put_code(P, pp, lane, -7); return; }
    }

    // ---- phase referencing (evd.cpp:738-749) ------------------------------
    const int mref = P.mini - 1;
    C2<T> zr;
    {
        C2<T> a = (mref < 32) ? z0 : z1;
        zr.x = __shfl_sync(0xffffffffu, a.x, mref & 31);
        zr.y = __shfl_sync(0xffffffffu, a.y, mref & 31);
    }
    const T zra2 = cabs2(zr);
    const C2<T> zru = (zra2 > T(0)) ? cscale(zr, rsqrt_t(zra2)) : cmk<T>(T(1), T(0));
    float2 ph0 = make_float2(0.f, 0.f), ph1 = make_float2(0.f, 0.f);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int i = lane + 32 * h;
        if (i >= n) continue;
        C2<T> z = h ? z1 : z0;
        T za2 = cabs2(z);
        C2<T> u = (za2 > T(0)) ? cscale(z, rsqrt_t(za2)) : cmk<T>(T(1), T(0));
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
#pragma unroll
        for (int h = 0; h < RS::H; ++h) {
            const int i = lane + 32 * h;
            const int ulim = (i < n) ? (stbas ? min(i + P.bw + 1, n) : n) : 0;
            const float2 pi = (i < n) ? phs[i] : make_float2(0.f, 0.f);
            cnt += max(ulim - i - 1, 0);
            // sum_j exp(i arg C_ij) ph_j over the row, then times conj(ph_i):
            // exp(i(arg C_ij - arg ph_i + arg ph_j)) summed over j > i
            T wr = T(0), wi = T(0);
#pragma unroll 1
            for (int cc = 0; cc < RS::CH; ++cc) {
                C2<T> cv[8];
                cp.load(h, cc, cv);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int j = 8 * cc + k;
                    if (j <= i || j >= ulim) continue;
                    const C2<T> c = cv[k];
                    const T ca2 = cabs2(c);
                    const C2<T> u = (ca2 > T(0)) ? cscale(c, rsqrt_t(ca2)) : cmk<T>(T(1), T(0));
                    const float2 pj = phs[j];
                    const C2<T> v = cmul(u, cmk<T>(T(pj.x), T(pj.y)));
                    wr += v.x;
                    wi += v.y;
                }
            }
            const C2<T> w = cmulc(cmk<T>(wr, wi), cmk<T>(T(pi.x), T(pi.y)));
            sr += w.x;
            si += w.y;
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


// Mixed form: pulls the Gamma record and tile information of pixel pp of P
// into L2 (one 128-byte line per lane), so the load of the next pixel of a
// warp finds them there.
__device__ __forceinline__ void prefetch_record(const KParams &P, long long pp, int lane)
{
    const long long loc = pp - P.cbase;
    const char *rec = reinterpret_cast<const char *>(P.cbuf) + loc * (long long)P.cstride * 4;
    const uintptr_t lo = reinterpret_cast<uintptr_t>(rec) & ~uintptr_t(127);
    const uintptr_t hi = reinterpret_cast<uintptr_t>(rec) + (size_t)P.cstride * 4;
    for (uintptr_t a = lo + 128u * (unsigned)lane; a < hi; a += 32u * 128u)
        asm volatile("prefetch.L2 [%0];" :: "l"(a));
    if (lane == 31) asm volatile("prefetch.L2 [%0];" :: "l"(P.cinfo + loc));
}

// Mixed form: Gamma of pixel pp was accumulated on the tensor cores
// (gram_box.cu) into a record of P.cstride floats; load it into the shared-
// memory matrix Cm of the warp and normalise it to coherence.  Record layout: dates padded to an even
// count and grouped in pairs; block (a, b), a <= b < DP, row-major over the
// upper triangle of pairs, holds Re, Im of Gamma_ij for (i, j) = (2a,2b),
// (2a,2b+1), (2a+1,2b), (2a+1,2b+1).  Returns the SHP count, or -1 when the
// pixel is finished (or handed to the FP64 path).
template <int NP, bool NORMALIZE = true>
__device__ int pixel_load_gamma(const KParams &P, long long pp, unsigned char *sm, int lane, C2<float> *Cm)
{
    using L = Lay<float, NP>;
    constexpr int LD = L::LD;
    const int n = P.nb;
    const long long plane = P.plane;
    for (int b = lane; b < n; b += 32) P.phase[b * plane + pp] = make_float2(0.f, 0.f);
    if (lane == 0) {
        P.tcorr[pp] = 0.f;
        P.comp[pp] = make_float2(0.f, 0.f);
    }
    const long long loc = pp - P.cbase;
    const int info = P.cinfo[loc];
    if (info == CI_CENTRE || info == CI_FEW) {
        if (P.status && lane == 0) P.status[pp] = (info == CI_CENTRE) ? 1 : 2;
        return -1;
    }
    if (info == CI_DEFER) {
        defer_fp64(P, pp, lane);
        return -1;
    }
    const float4 *rec4 =
        reinterpret_cast<const float4 *>(reinterpret_cast<const float *>(P.cbuf) + loc * (long long)P.cstride);
    const int dp = (n + 1) >> 1, nblk = dp * (dp + 1) / 2;
    // blocks t = 0 .. nblk-1, row-major over the upper triangle of pairs
    // (pair row a holds blocks (a, a) .. (a, dp-1)).  Counted from the last
    // block, t' = nblk-1-t lies in pair row a = dp-1-r for r(r+1)/2 <= t' <
    // (r+1)(r+2)/2, at column b = dp-1-(t' - r(r+1)/2).  Each lane loads
    // four blocks before it stores any.
    for (int t0 = 0; t0 < nblk; t0 += 128) {
        float4 u[4], v[4];
#pragma unroll
        for (int s4 = 0; s4 < 4; ++s4) {
            const int t = t0 + lane + 32 * s4;
            u[s4] = v[s4] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (t < nblk) {
                u[s4] = __ldg(rec4 + 2 * t);
                v[s4] = __ldg(rec4 + 2 * t + 1);
            }
        }
#pragma unroll
        for (int s4 = 0; s4 < 4; ++s4) {
            const int t = t0 + lane + 32 * s4;
            if (t >= nblk) continue;
            const int tr = nblk - 1 - t;
            const int r = (int)((sqrtf((float)(8 * tr + 1)) - 1.f) * 0.5f);
            const int a = dp - 1 - r, b = dp - 1 - (tr - r * (r + 1) / 2);
            const int i0 = 2 * a, i1 = 2 * a + 1, j0 = 2 * b, j1 = 2 * b + 1;
            if (j0 < n) Cm[i0 * LD + j0] = cmk<float>(u[s4].x, u[s4].y);
            if (j1 < n) Cm[i0 * LD + j1] = cmk<float>(u[s4].z, u[s4].w);
            if (i1 < n && j0 >= i1) Cm[i1 * LD + j0] = cmk<float>(v[s4].x, v[s4].y);
            if (j1 < n) Cm[i1 * LD + j1] = cmk<float>(v[s4].z, v[s4].w);
        }
    }
    __syncwarp();
    if (!NORMALIZE) return info;
    return gamma_to_coherence<float, NP>(P, pp, Cm, sm, lane) ? info : -1;
}

// rows of the coherence matrix C in shared memory (ld NP+1, full storage)
// into the row policy cp (every lane calls it together)
template <int NP, typename CP, typename T>
__device__ void rows_from_smem(const CP &cp, const C2<T> *A, int lane)
{
#pragma unroll
    for (int h = 0; h < RowShape<NP>::H; ++h) {
        const int i = lane + 32 * h;
#pragma unroll 1
        for (int c = 0; c < RowShape<NP>::CH; ++c) {
            C2<T> v[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) v[k] = (i < NP) ? A[i * (NP + 1) + 8 * c + k] : cmk<T>(T(0), T(0));
            cp.store(h, c, v);
        }
    }
    cp.fence();
    __syncwarp();
}

// Gamma (upper triangle and diagonal of G, ld NP+1) to coherence rows in
// the row policy cp, for NP <= 32 (one row per lane): the rule of
// gamma_to_coherence (C_ij = Gamma_ij / sqrt(P_i P_j) scaled in the same
// order, lower triangle by conjugation, unit diagonal), with rows and
// columns >= n set to zero.  Returns false (and writes the failure code)
// when a result is not finite.
template <int NP, typename CP>
__device__ bool rows_coherence(const KParams &P, long long pp, const C2<float> *G, unsigned char *sm,
                               const CP &cp, int lane, float *cfro)
{
    static_assert(NP <= 32 && NP % 8 == 0, "one row per lane");
    constexpr int LD = NP + 1;
    float *yv = reinterpret_cast<float *>(sm + Lay<float, NP>::yy);
    const int n = P.nb;
    bool bad = false;
    if (lane < n) {
        const float Pi = G[lane * LD + lane].x;
        bad = !(Pi > 0.f) || !isfinite(Pi);
        yv[lane] = 1.f / sqrtf(Pi);
    }
    bad = __any_sync(0xffffffffu, bad);
    __syncwarp();
    float fs = 0.f;                    // |C|_F^2, summed as the solver's own pass would
    if (!bad) {
        const float ri = (lane < n) ? yv[lane] : 0.f;
#pragma unroll 1
        for (int c = 0; c < NP / 8; ++c) {
            const float4 ya = *reinterpret_cast<const float4 *>(yv + 8 * c);
            const float4 yb = *reinterpret_cast<const float4 *>(yv + 8 * c + 4);
            const float yj[8] = {ya.x, ya.y, ya.z, ya.w, yb.x, yb.y, yb.z, yb.w};
            C2<float> v[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const int j = 8 * c + k;
                C2<float> e = cmk<float>(0.f, 0.f);
                if (lane < n && j < n) {
                    if (j > lane) {
                        e = cscale(G[lane * LD + j], ri * yj[k]);
                    } else if (j < lane) {
                        // the conjugate of row j's entry, scaled in its order
                        e = cconj(cscale(G[j * LD + lane], yj[k] * ri));
                    } else {
                        e = cmk<float>(1.f, 0.f);
                    }
                    bad |= !isfinite(e.x) || !isfinite(e.y);
                    fs += cabs2(e);
                }
                v[k] = e;
            }
            cp.store(0, c, v);
        }
        cp.fence();
        bad = __any_sync(0xffffffffu, bad);
    }
    *cfro = sqrtf(warp_sum(fs));
    __syncwarp();
    if (bad) {
        // non-finite coherence: the first eigen call is reported as failed
        put_code(P, pp, lane, (P.semantics != SEM_PL && P.method != M_MLE) ? -6 : -1);
        return false;
    }
    return true;
}

// taddr: the warp's tensor-memory rows when CInTmem<T, NP> or
// CRowsTmemF<T, NP> (C is formed in shared memory, then moved there before
// the solve reuses that memory)
template <typename T, int NP>
__device__ void process_pixel(const KParams &P, long long pp, unsigned char *sm, int lane, uint32_t taddr = 0)
{
    const int npix = pixel_coherence<T, NP>(P, pp, sm, lane);
    if (npix < 0) return;
    const C2<T> *Cm = reinterpret_cast<const C2<T> *>(sm + CmOffset<T, NP>::value);
    if constexpr (CInTmem<T, NP>::value) {
        const CRowsTmemD<NP> cp{taddr};
        rows_from_smem<NP>(cp, Cm, lane);
        pixel_solve<T, NP>(P, pp, sm, lane, npix, cp);
    } else if constexpr (CRowsTmemF<T, NP>::value) {
        const CRowsTmem<NP> cp{taddr};
        rows_from_smem<NP>(cp, Cm, lane);
        pixel_solve<T, NP>(P, pp, sm, lane, npix, cp);
    } else {
        const CRowsSmem<T, NP> cp{const_cast<C2<T> *>(Cm), lane};
        pixel_solve<T, NP>(P, pp, sm, lane, npix, cp);
    }
}

}  // namespace fpl
