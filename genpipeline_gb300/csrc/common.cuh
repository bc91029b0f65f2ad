// common.cuh -- shared definitions of the gbsimp CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbsimp.h"

namespace gbs {

// Element-local node a sits at corner (cx, cy, cz) of its element; reference order of
// genpipeline/topology/simp_solver.py:256-266.
__host__ __device__ constexpr int corner_x(int a) { return (a == 1 || a == 2 || a == 5 || a == 6) ? 1 : 0; }
__host__ __device__ constexpr int corner_y(int a) { return (a == 2 || a == 3 || a == 6 || a == 7) ? 1 : 0; }
__host__ __device__ constexpr int corner_z(int a) { return a >= 4 ? 1 : 0; }

// Element stiffness passed BY VALUE as a kernel parameter: kernel parameters live in a
// constant bank, so with fully unrolled loops every Ke entry is an FFMA/DFMA operand read
// straight from the constant cache, with no load instruction and no shared memory.
struct KeF {
    float k[576];
};
struct KeD {
    double k[576];
};

// Stiffness law (gbsimp_law) in the arithmetic type of a kernel.
template <typename T>
struct Law {
    int kind;  // 0 ref: e0*max(x,xmin)^p ; 1 modified: emin + x^p (e0-emin)
    int pint;  // penal when it is an integer 1..4, else -1
    T penal, e0, emin, xmin;
};

template <typename T>
Law<T> make_law(const gbsimp_law &l) {
    Law<T> r;
    r.kind = l.kind;
    r.penal = (T)l.penal;
    r.e0 = (T)l.e0;
    r.emin = (T)l.emin;
    r.xmin = (T)l.xmin;
    r.pint = -1;
    for (int i = 1; i <= 4; ++i)
        if (l.penal == (double)i) r.pint = i;
    return r;
}

// x^n for n in 0..4 by multiplication, else pow(x, p).
__device__ __forceinline__ double powp(double x, int n, double p) {
    switch (n) {
        case 0: return 1.0;
        case 1: return x;
        case 2: return x * x;
        case 3: return x * x * x;
        case 4: return (x * x) * (x * x);
        default: return pow(x, p);
    }
}
__device__ __forceinline__ float powp(float x, int n, float p) {
    switch (n) {
        case 0: return 1.0f;
        case 1: return x;
        case 2: return x * x;
        case 3: return x * x * x;
        case 4: return (x * x) * (x * x);
        default: return powf(x, p);
    }
}

// E(x) of one element.
template <typename T>
__device__ __forceinline__ T modulus(const Law<T> &L, T x) {
    if (L.kind == 0) {
        T xm = x > L.xmin ? x : L.xmin;
        return L.e0 * powp(xm, L.pint, L.penal);
    }
    return L.emin + powp(x, L.pint, L.penal) * (L.e0 - L.emin);
}

// dE/dx of one element; law 0 evaluates it at the floored density, as the reference does
// (simp_solver.py:218).
template <typename T>
__device__ __forceinline__ T dmodulus(const Law<T> &L, T x) {
    const int n1 = L.pint >= 1 ? L.pint - 1 : -1;
    if (L.kind == 0) {
        T xm = x > L.xmin ? x : L.xmin;
        return L.e0 * L.penal * powp(xm, n1, L.penal - (T)1);
    }
    return L.penal * powp(x, n1, L.penal - (T)1) * (L.e0 - L.emin);
}

// Warp / block sums in FP64 (fixed shuffle order => deterministic).
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Sums v over the block (1-D, 2-D or 3-D; the thread count must be a multiple of 32); the
// result is valid in the thread with linear id 0. scratch: >= 32 doubles.
__device__ __forceinline__ double block_sum(double v, double *scratch) {
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, warp = tid >> 5;
    const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (warp == 0) {
        r = lane < nw ? scratch[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// K block sums at once, with one pair of barriers (each value follows the tree of
// block_sum, so the results are the same); valid in thread 0. scratch: 32 K doubles.
template <int K>
__device__ __forceinline__ void block_sum_n(double (&v)[K], double *scratch) {
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, warp = tid >> 5;
    const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) scratch[32 * k + warp] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double r = 0.0;
        if (warp == 0) {
            r = lane < nw ? scratch[32 * k + lane] : 0.0;
            r = warp_sum(r);
        }
        v[k] = r;
    }
}

// Double-float arithmetic: a value hi + lo held as two FP32 numbers, about 44-48 significant
// bits (Dekker 1971; Knuth's exact two-sum for the add). Used for the sums and the scalar
// recurrence of the one-kernel PCG iteration, which sit on its critical path: on this part an
// FP64 division takes about 550 cycles and an FP64 add or fma about 64, a double-float add
// about 30. The add is commutative, so butterfly reductions leave every lane with the same
// value.
struct df32 {
    float hi, lo;
};
__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float hi = __fadd_rn(s, e);
    const float lo = __fsub_rn(e, __fsub_rn(hi, s));
    return df32{hi, lo};
}
__device__ __forceinline__ double df_value(df32 a) { return (double)a.hi + (double)a.lo; }
__host__ __device__ __forceinline__ df32 df_from(double v) {
    const float hi = (float)v;
    return df32{hi, (float)(v - (double)hi)};
}
__device__ __forceinline__ df32 df_neg(df32 a) { return df32{-a.hi, -a.lo}; }
// (a + b) renormalised, for |a| >= |b| (Dekker's fast two-sum).
__device__ __forceinline__ df32 df_renorm(float a, float b) {
    const float s = __fadd_rn(a, b);
    return df32{s, __fsub_rn(b, __fsub_rn(s, a))};
}
// Product: the rounding error of a.hi * b.hi comes exactly from one fma (Dekker's product).
__device__ __forceinline__ df32 df_mul(df32 a, df32 b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_renorm(p, e);
}
// Quotient by long division: the FP32 quotient of the leading parts, corrected once by the
// quotient of the remainder a - q b.
__device__ __forceinline__ df32 df_div(df32 a, df32 b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const df32 r = df_add(a, df_neg(df_mul(df32{q1, 0.0f}, b)));
    return df_renorm(q1, __fdiv_rn(r.hi, b.hi));
}

// K block sums in double-float with one pair of barriers; valid in thread 0. scratch: 32 K
// float2.
template <int K>
__device__ __forceinline__ void block_sum_df(df32 (&v)[K], float2 *scratch) {
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    const int lane = tid & 31, warp = tid >> 5;
    const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v[k] = df_add(v[k], df32{__shfl_xor_sync(0xffffffffu, v[k].hi, o), __shfl_xor_sync(0xffffffffu, v[k].lo, o)});
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) scratch[32 * k + warp] = make_float2(v[k].hi, v[k].lo);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        df32 r{0.0f, 0.0f};
        if (warp == 0) {
            if (lane < nw) r = df32{scratch[32 * k + lane].x, scratch[32 * k + lane].y};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                r = df_add(r, df32{__shfl_xor_sync(0xffffffffu, r.hi, o), __shfl_xor_sync(0xffffffffu, r.lo, o)});
        }
        v[k] = r;
    }
}

// Division of a grid index n < 2^31 by a fixed divisor 1 <= d < 2^31 as a multiply-high, an add
// and a shift (Granlund and Montgomery 1994, round-up method): with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (umulhi(n, m) + n) >> l for every n < 2^32 when
// the sum is formed in 33 bits; for n < 2^31 it fits in 32. Replaces the 64-bit divisions of
// the element and node index decompositions, which compile to a long call sequence.
struct FastDiv {
    uint32_t d, m, l;
};
inline FastDiv fast_div(uint32_t d) {
    uint32_t l = 0;
    while (l < 31 && (1u << l) < d) ++l;
    const uint64_t m = (((uint64_t)1 << 32) * (((uint64_t)1 << l) - d)) / d + 1;
    return FastDiv{d, (uint32_t)m, l};
}
__host__ __device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
#ifdef __CUDA_ARCH__
    return (__umulhi(n, f.m) + n) >> f.l;
#else
    return (uint32_t)((((uint64_t)n * f.m) >> 32) + n) >> f.l;
#endif
}
// (i, j, k) of the row-major index n of an (a, b, c) box, k fastest: by = fast_div(b), bc = fast_div(c).
__host__ __device__ __forceinline__ void unflatten3(uint32_t n, const FastDiv &fb, const FastDiv &fc, int &i, int &j,
                                                    int &k) {
    const uint32_t q = fdiv(n, fc);
    k = (int)(n - q * fc.d);
    const uint32_t p = fdiv(q, fb);
    j = (int)(q - p * fb.d);
    i = (int)p;
}

// Unnormalised double-float values for the element products of the outer residual and of the
// sensitivities (fp64.cu, pcg.cu): a value is h + l. Every add of leading parts is an exact
// two-sum whose rounding error moves into l, every product takes the error of its leading
// product from one fma (Dekker), and the l parts are carried with plain FP32 adds and never
// renormalised. The leading parts are thus exact and the only rounding is that of the l chain,
// about 2^-46 of the magnitudes that enter a butterfly or a row. Exact as long as no leading
// part or rounding error falls below the FP32 normal range (|values| above about 1e-30).
struct ddv {
    float h, l;
};
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ ddv dd_of(double v) {
    const float h = __double2float_rn(v);
    return ddv{h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ double dd_value(ddv a) { return (double)a.h + (double)a.l; }
// (double)x from the bits of a normal FP32 x (exponent rebiased, mantissa widened); zero,
// subnormals, infinities and NaN take the conversion instruction.
// The rare paths below are calls, so that the compiler branches around their conversion
// instructions instead of predicating them into every evaluation.
static __device__ __noinline__ double f2d_slow(float x) { return (double)x; }
__device__ __forceinline__ double f2d(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned e = (b >> 23) & 0xffu;
    if ((b & 0x7fffffffu) == 0u) return __longlong_as_double((long long)((unsigned long long)(b >> 31) << 63));
    if (e == 0u || e == 0xffu) return f2d_slow(x);
    return __longlong_as_double((long long)(((unsigned long long)(b >> 31) << 63) |
                                            ((unsigned long long)(e + 896u) << 52) |
                                            ((unsigned long long)(b & 0x7fffffu) << 29)));
}
// dd_of(v) from the bits of v with integer operations, off the FP64 pipe (whose conversions
// run far below its add rate on this part): h = v rounded to 24 bits (nearest, ties to even)
// as an integer add on the bit pattern, v - h = (bits(v) - bits(h)) units of 2^(e - 1075) (the
// difference of the patterns counts mantissa units across a binade carry too), rounded to
// FP32 by the integer conversion and scaled exactly. Values with |v| outside [2^-70, 2^100],
// and zero, subnormals, infinities and NaN, take dd_of.
static __device__ __noinline__ ddv dd_of_slow(double v) { return dd_of(v); }
__device__ __forceinline__ ddv dd_split(double v) {
    const long long b = __double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);
    if ((b & 0x7fffffffffffffffLL) == 0) return ddv{0.0f, 0.0f};
    if (e < 1023 - 70 || e > 1023 + 100) return dd_of_slow(v);
    const long long rb = (b + ((1LL << 28) - 1) + ((b >> 29) & 1)) & ~((1LL << 29) - 1);
    const int eh = (int)((rb >> 52) & 0x7ff);
    const unsigned sign = (unsigned)((unsigned long long)b >> 63) << 31;
    const float h = __uint_as_float(sign | ((unsigned)(eh - 1023 + 127) << 23) | (unsigned)((rb >> 29) & 0x7fffff));
    const int d = (int)(b - rb);  // |d| <= 2^28: the remainder in units of 2^(e - 1075), sign of |v| - |h|
    const float scale = __uint_as_float((unsigned)(e - 1075 + 127) << 23);
    const float l = __fmul_rn(__int2float_rn(d), scale);
    return ddv{h, sign ? -l : l};
}
__device__ __forceinline__ ddv dd_add(ddv a, ddv b) {
    float s, e;
    two_sum(a.h, b.h, s, e);
    return ddv{s, __fadd_rn(__fadd_rn(a.l, b.l), e)};
}
// (a, b) <- (a + b, b - a): one stage of the forward Walsh-Hadamard transform
__device__ __forceinline__ void dd_fwd(ddv &a, ddv &b) {
    float s, e, d, g;
    two_sum(a.h, b.h, s, e);
    two_sum(b.h, -a.h, d, g);
    const ddv lo{s, __fadd_rn(__fadd_rn(a.l, b.l), e)};
    b = ddv{d, __fadd_rn(__fsub_rn(b.l, a.l), g)};
    a = lo;
}
// (a, b) <- (a - b, a + b): one stage of the inverse transform
__device__ __forceinline__ void dd_inv(ddv &a, ddv &b) {
    float s, e, d, g;
    two_sum(a.h, -b.h, d, g);
    two_sum(a.h, b.h, s, e);
    const ddv hi{s, __fadd_rn(__fadd_rn(a.l, b.l), e)};
    a = ddv{d, __fadd_rn(__fsub_rn(a.l, b.l), g)};
    b = hi;
}
// (ch + cl) (q.h + q.l), the product of the low parts dropped
__device__ __forceinline__ ddv dd_mul(float ch, float cl, ddv q) {
    const float p = __fmul_rn(ch, q.h);
    float e = __fmaf_rn(ch, q.h, -p);
    e = __fmaf_rn(ch, q.l, e);
    e = __fmaf_rn(cl, q.h, e);
    return ddv{p, e};
}

constexpr int kModalNnz = 45;

// Modal form of the isotropic cube element (see apply_modal.cuh). Sparsity pattern of Km in (mode*3 + component) indices (derived from the quadrature
// element; capi.cu checks that the installed Ke has no entry outside it).
__host__ __device__ constexpr int modal_row(int i) {
    constexpr int r[kModalNnz] = {3,  3,  4,  4,  5,  5,  5,  6,  6,  7,  7,  7,  8,  8,  9,  9,  9,  10, 10, 11, 11, 12, 12,
                                  12, 13, 13, 14, 14, 15, 15, 16, 16, 16, 17, 17, 18, 18, 19, 19, 20, 20, 20, 21, 22, 23};
    return r[i];
}
__host__ __device__ constexpr int modal_col(int i) {
    constexpr int c[kModalNnz] = {3, 14, 4,  8,  5,  7,  12, 6,  13, 5,  7,  12, 4,  8,  9,  16, 20, 10, 15, 11, 18, 5, 7,
                                  12, 6, 13, 3, 14, 10, 15, 9,  16, 20, 17, 19, 11, 18, 17, 19, 9,  16, 20, 21, 22, 23};
    return c[i];
}

// Km splits into 11 independent blocks of 1-3 (mode, component) indices; row r only reads
// columns of its own block, so r = Km q can overwrite q block by block.
constexpr int kModalBlocks = 11;
__host__ __device__ constexpr int modal_block(int b, int a) {
    constexpr int m[kModalBlocks][3] = {{3, 14, -1},  {4, 8, -1},   {5, 7, 12},   {6, 13, -1},
                                        {9, 16, 20},  {10, 15, -1}, {11, 18, -1}, {17, 19, -1},
                                        {21, -1, -1}, {22, -1, -1}, {23, -1, -1}};
    return m[b][a];
}
__host__ __device__ constexpr int modal_block_of(int r) {
    for (int b = 0; b < kModalBlocks; ++b)
        for (int a = 0; a < 3; ++a)
            if (modal_block(b, a) == r) return b;
    return -1;
}
__host__ __device__ constexpr bool modal_blocks_closed() {
    for (int i = 0; i < kModalNnz; ++i)
        if (modal_block_of(modal_row(i)) < 0 || modal_block_of(modal_row(i)) != modal_block_of(modal_col(i)))
            return false;
    return true;
}
static_assert(modal_blocks_closed(), "every Km entry must lie inside one block");
__host__ __device__ constexpr bool modal_row_first(int i) { return i == 0 || modal_row(i - 1) != modal_row(i); }

// By the cube's symmetry the 45 coefficients take at most 8 distinct values for any isotropic
// material (fewer for some Poisson ratios, e.g. 7 at nu = 0.3); entry i has the value of class
// modal_class(i). capi.cu checks this for the installed Ke.
constexpr int kModalClasses = 8;
__host__ __device__ constexpr int modal_class(int i) {
    constexpr int k[kModalNnz] = {0, 0, 0, 0, 1, 2, 2, 0, 0, 2, 1, 2, 0, 0, 3, 4, 4, 5, 6, 5, 6, 2, 2,
                                  1, 0, 0, 0, 0, 6, 5, 4, 3, 4, 5, 6, 6, 5, 6, 5, 4, 4, 3, 7, 7, 7};
    return k[i];
}

// The class values, each duplicated into both lanes of a float2 (packed FP32x2 operands: one
// thread works on two elements at once).
struct ModalK {
    float2 c[kModalClasses];
};
struct ModalKD {
    double v[kModalNnz];
};
// The same as double-float pairs (h + l = the FP64 value to 2^-48).
struct ModalKDD {
    float h[kModalNnz], l[kModalNnz];
};

}  // namespace gbs

// ---- library-internal host helpers (capi.cu) -------------------------------------------
struct gbsimp_ctx {
    int device;
    double ke[576];
    gbs::KeF kef;
    gbs::KeD ked;
    bool translation_free;  // Ke annihilates rigid translations (quadrature Ke: yes)
    float ke_diag_f[24];
    double ke_diag_d[24];
    int num_sms;
    int smem_per_sm;        // shared memory per SM (bytes)
    bool modal_ok;          // Ke has the modal sparsity of an isotropic cube element
    gbs::ModalK km;         // its 45 modal coefficients (Km / 64)
    gbs::ModalKD kmd;       // the same in FP64
    unsigned ke_version;    // bumped by every set_ke (keys the graph cache)
    void *graphs;           // gbs::GraphCache* (pcg.cu): instantiated device-loop graphs
};

namespace gbs {
int set_error(int code, const char *fmt, ...);
int cuda_error(cudaError_t e, const char *what);
void count_launches(int n);
void set_capturing(bool on);
void *graph_cache_create();
void graph_cache_destroy(void *gc);
}  // namespace gbs

#define GBS_CUDA_TRY(call)                                           \
    do {                                                             \
        cudaError_t _e = (call);                                     \
        if (_e != cudaSuccess) return gbs::cuda_error(_e, #call);    \
    } while (0)

#define GBS_LAUNCH_CHECK(what)                                       \
    do {                                                             \
        gbs::count_launches(1);                                      \
        cudaError_t _e = cudaGetLastError();                         \
        if (_e != cudaSuccess) return gbs::cuda_error(_e, what);     \
    } while (0)
