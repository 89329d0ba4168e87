// Shared definitions for the GB300 gravity library.
//
// Every translation unit is compiled with --fmad=false: a product followed
// by a sum is rounded twice unless the code calls fma() explicitly.  The
// bit-exact paths rely on this to reproduce the reference's C arithmetic;
// the fast paths spell out the fma() calls they want.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <string.h>

#include "abie_gb300.h"

namespace abie {

// Compact source record: predicted position and G*m of one massive body.
struct __align__(32) Src {
    double x, y, z, gm;
};

// Per-call error reporting (host side), defined in abi.cu.
void set_error(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

#define ABIE_CUDA(call)                                                   \
    do {                                                                  \
        cudaError_t _e = (call);                                          \
        if (_e != cudaSuccess) return ::abie::cuda_fail(_e, #call);       \
    } while (0)

// Device pair term for the fast FP64 form: G m / r^3 from r^2 with no FP64
// instruction at all.
//
// Seed: r2 truncated to 23 mantissa bits as a float, its single-precision
// reciprocal square root y truncated to a 21-bit significand m, so that
// y = m 2^E, y^2 = m^2 2^2E (m^2 < 2^42) and y^3 = m^3 2^3E (m^3 < 2^63)
// exactly, in 64-bit integers.  With e = 1 - r2 y^2 (|e| < 2^-18),
//     r2^(-3/2) = y^3 (1 - e)^(-3/2) = y^3 (1 + k),  k = 3/2 e + 15/8 e^2 + 35/16 e^3 + O(e^4).
// Everything is integer arithmetic on fixed-point numbers with 62
// fractional bits: e from the high word of the product of r2's 53-bit
// significand and m^2, e^2 and e^3 in FP32, F = (1 + k) 2^62, the high word
// of m^3 F, the high word of its product with the significand of G m, and
// the result assembled as a double, rounded half up on the first dropped
// bit.  The intermediate steps truncate, but at 2^-60 relative and below,
// so the result is unbiased and within about half an ulp: a C restatement
// of r2_int and these operations over 2 million random separations (each
// component 1e-9 .. 2e4 or zero) and G m in [1e-12, 1e2], with the FP32
// seed perturbed by up to 2^-22, is at most 0.53 ulp from the exact
// G m |d|^-3, mean signed error +0.001 ulp (truncating the last step
// instead: at most 1.03 ulp, every factor 0.5 ulp small on average; from
// a double r2, as gm_inv_r3 takes it, r2's own rounding adds up to 0.75
// ulp).  r2 = 0 (a body and itself) gives a finite value, so the
// caller's 0 * w is exactly zero.  r2 must lie within the FP32 exponent
// range.  The FP64 pipe is left to the separations, r2 and the sums.
__device__ __forceinline__ int clamp_exp_f32(int hi_rebased)
{
    // keep the single-precision exponent in [1, 254]
    return min(max(hi_rebased, 1 << 20), (254 << 20) | 0xFFFFF);
}

__device__ __forceinline__ double f32_bits_to_f64(int fb)
{
    // exact conversion of a positive normal float given by its bits
    return __hiloint2double((fb >> 3) + ((1023 - 127) << 20), fb << 29);
}

__device__ __forceinline__ float f64_to_f32_trunc(double v)
{
    // |v| truncated to 20 mantissa bits, as a float (sign dropped)
    int hi = __double2hiint(v) & 0x7FFFFFFF;
    return __int_as_float(clamp_exp_f32(hi - ((1023 - 127) << 20)) << 3);
}

__device__ __forceinline__ float f64_to_f32_trunc23(double v)
{
    // |v| truncated to 23 mantissa bits, as a float (sign dropped)
    int hi = __double2hiint(v) & 0x7FFFFFFF;
    unsigned lo = (unsigned)__double2loint(v);
    return __uint_as_float(((unsigned)clamp_exp_f32(hi - ((1023 - 127) << 20)) << 3) | (lo >> 29));
}

__device__ __forceinline__ double f32_to_f64_signed(float f)
{
    // exact conversion of a normal (or zero) float, sign kept
    unsigned b = __float_as_uint(f);
    unsigned sgn = b & 0x80000000u;
    b &= 0x7FFFFFFFu;
    if (b == 0u) return 0.0;
    return __hiloint2double((int)(((b >> 3) + ((1023 - 127) << 20)) | sgn), (int)(b << 29));
}

// The core on r2 = Mr 2^Er, Mr a 64-bit significand with its top bit set
// (or 0 for r2 = 0), in two parts: r^-3 as a normalised 64-bit significand
// Wn (top bit set) with exponent eW, then its product with G m, so that a
// pair evaluated for both of its bodies (the symmetric force) shares the
// first part.
__device__ __forceinline__ void inv_r3_core(unsigned long long Mr, int Er, unsigned long long &Wn,
                                            int &eW)
{
    typedef unsigned long long ull;
    // seed: r2 truncated to 24 bits as a float, its rsqrtf cut to 21 bits
    const int fe = min(max(Er + 63 + 127, 1), 254);
    const float r2f = __uint_as_float(Mr ? (((unsigned)fe << 23) | (unsigned)((Mr >> 40) & 0x7FFFFFull))
                                         : (1u << 23));
    const float yf = rsqrtf(r2f);
    const unsigned yb = __float_as_uint(yf);
    const ull m = (ull)(((yb & 0x7FFFFFu) | 0x800000u) >> 3);
    const int E = (int)(yb >> 23) - 147;  // y = m 2^E
    const ull m2 = m * m;                 // [2^40, 2^42)
    // e 2^62 = 2^62 - r2 m^2 2^(2E + 62); the high word of Mr (m^2 2^22)
    // is Mr m^2 / 2^42
    const ull Phi = __umul64hi(Mr, m2 << 22);
    const int s2 = -(104 + Er + 2 * E);  // 0..2 for r2 in range
    long long eh = 0;                    // r2 = 0: any finite value
    if (Mr && s2 >= 0 && s2 < 64) eh = (long long)((1ull << 62) - (Phi >> s2));
    else if (Mr && s2 < 0 && s2 > -3) eh = (long long)((1ull << 62) - (Phi << (-s2)));
    // e as a float (truncated) for the FP32 terms
    const ull ae = (ull)(eh < 0 ? -eh : eh);
    const int lze = __clzll((long long)ae);
    const unsigned fb = ae ? (((unsigned)(128 - lze) << 23) | (unsigned)(((ae << lze) >> 40) & 0x7FFFFFull)) : 0u;
    const float ef = __uint_as_float(fb | (eh < 0 ? 0x80000000u : 0u));
    // 15/8 e^2 + 35/16 e^3 (non-negative) to the same fixed point
    const float q = ef * ef * fmaf(2.1875f, ef, 1.875f);
    const unsigned qb = __float_as_uint(q);
    const int eq = (int)(qb >> 23);
    const ull mq = (ull)((qb & 0x7FFFFFu) | 0x800000u);
    ull qh = eq >= 88 ? (mq << min(eq - 88, 40)) : ((88 - eq) < 64 ? (mq >> (88 - eq)) : 0ull);
    qh = qb ? qh : 0ull;
    const long long kh = eh + (eh >> 1) + (long long)qh;  // k 2^62
    const ull F = (1ull << 62) + (ull)kh;                 // (1 + k) 2^62
    const ull m3 = m2 * m;                                // [2^60, 2^63)
    const ull W = __umul64hi(m3, F);                      // m^3 (1 + k) 2^-2
    const int lz = __clzll((long long)W);
    Wn = W << lz;
    eW = 3 * E - lz;
}

__device__ __forceinline__ double gm_times_inv_r3(unsigned long long Wn, int eW, double gm)
{
    typedef unsigned long long ull;
    const ull gb = (ull)__double_as_longlong(gm);
    const int eg = (int)((gb >> 52) & 0x7FF);
    const ull Mg = (gb & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const ull Z = __umul64hi(Mg << 11, Wn);
    const int lz2 = __clzll((long long)Z);
    const ull Zn = Z << lz2;
    const int be = min(max(eg + eW - lz2 + 66, 1), 2046);
    // round half up on the first dropped bit: adding it to the bit pattern
    // carries a full significand into the exponent (truncating instead
    // would make every factor 0.5 ulp small on average)
    const ull bits = ((ull)be << 52) | ((Zn >> 11) & 0xFFFFFFFFFFFFFull);
    return __longlong_as_double((long long)(bits + ((Zn >> 10) & 1ull)));
}

__device__ __forceinline__ double gm_inv_r3_int(unsigned long long Mr, int Er, double gm)
{
    unsigned long long Wn;
    int eW;
    inv_r3_core(Mr, Er, Wn, eW);
    return gm_times_inv_r3(Wn, eW, gm);
}

__device__ __forceinline__ double gm_inv_r3(double r2, double gm)
{
    typedef unsigned long long ull;
    const ull rb = (ull)__double_as_longlong(r2);
    const int er = (int)((rb >> 52) & 0x7FF);
    const ull Mr = er ? (((rb & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 11) : 0ull;
    return gm_inv_r3_int(Mr, er - 1075 - 11, gm);
}

// d^2 for a double d as S 2^e2, S = the high word of (M 2^11)^2 (top bit set)
// for d's 53-bit significand M; S = 0 for d = 0 (or subnormal).
__device__ __forceinline__ void square_int(double d, unsigned long long &S, int &e2)
{
    typedef unsigned long long ull;
    const ull b = (ull)__double_as_longlong(d);
    const int ex = (int)((b >> 52) & 0x7FF);
    const ull M = ((b & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 11;
    S = ex ? __umul64hi(M, M) : 0ull;
    e2 = ex ? 2 * (ex - 1075) + 42 : -100000;
}

// r2 = dx^2 + dy^2 + dz^2 as Mr 2^Er (64-bit significand, top bit set, or
// 0), all integer: the three squares' high words aligned to the largest
// exponent and added (truncating; about 2^-61 relative).
__device__ __forceinline__ void r2_int(double dx, double dy, double dz, unsigned long long &Mr,
                                       int &Er)
{
    typedef unsigned long long ull;
    ull Sx, Sy, Sz;
    int ex, ey, ez;
    square_int(dx, Sx, ex);
    square_int(dy, Sy, ey);
    square_int(dz, Sz, ez);
    const int K = max(ex, max(ey, ez));
    const int hx = K - ex, hy = K - ey, hz = K - ez;
    ull T = (hx < 64 ? (Sx >> hx) : 0ull) >> 2;
    T += (hy < 64 ? (Sy >> hy) : 0ull) >> 2;
    T += (hz < 64 ? (Sz >> hz) : 0ull) >> 2;
    const int lz = __clzll((long long)T);
    Mr = T ? (T << lz) : 0ull;
    Er = K + 2 - lz;
}

// 1/sqrt(x) for positive normal x and 1/x for normal x of either sign,
// |x| within the single-precision exponent range (2^-126 < |x| < 2^127),
// each a few ulp from the exact value
// in 3 FP64 instructions.  Same construction as gm_inv_r3: a seed y = m 2^E
// with a 21-bit significand from the FP32 rsqrtf / rcp, assembled into a
// double by integer instructions, then one correction with its quadratic
// and cubic terms in FP32:
//   x^(-1/2) = y (1 - e)^(-1/2) = y (1 + e/2 + 3/8 e^2 + 5/16 e^3),  e = 1 - x y^2
//   x^(-1)   = y (1 - e)^(-1)   = y (1 + e + e^2 + e^3),             e = 1 - x y
__device__ __forceinline__ double seed_to_f64(float yf, unsigned long long &m, int &E)
{
    const unsigned yb = __float_as_uint(yf);
    m = (unsigned long long)(((yb & 0x7FFFFFu) | 0x800000u) >> 3);  // 21 bits
    E = (int)(yb >> 23) - 147;                                        // y = m 2^E
    const unsigned long long bits = ((unsigned long long)(long long)(20 + E + 1023) << 52) |
                                    ((m << 32) & 0xFFFFFFFFFFFFFull);
    return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ float signed_trunc23(double e)
{
    float ef = f64_to_f32_trunc23(e);
    return (__double2hiint(e) < 0) ? -ef : ef;
}

__device__ __forceinline__ double inv_sqrt_fast(double x)
{
    unsigned long long m;
    int E;
    const double y = seed_to_f64(rsqrtf(f64_to_f32_trunc23(x)), m, E);
    const unsigned long long m2 = m * m;  // [2^40, 2^42): y^2 exact
    const int p2 = 40 + (int)(m2 >> 41);
    const double t = __longlong_as_double((long long)(
        ((unsigned long long)(long long)(p2 + 2 * E + 1023) << 52) | ((m2 << (52 - p2)) & 0xFFFFFFFFFFFFFull)));
    const double e = fma(-x, t, 1.0);
    const float ef = signed_trunc23(e);
    const float q = ef * ef * fmaf(0.3125f, ef, 0.375f);
    const double k = fma(e, 0.5, f32_to_f64_signed(q));
    return fma(y, k, y);
}

// 1/x of either sign: the construction runs on |x| and the sign bit is
// copied back by integer instructions (the Kepler iteration's radius
// function can turn negative far from its root).
__device__ __forceinline__ double rcp_fast(double x)
{
    const long long sgn = __double_as_longlong(x) & (long long)0x8000000000000000ull;
    const double ax = __longlong_as_double(__double_as_longlong(x) ^ sgn);
    unsigned long long m;
    int E;
    const double y = seed_to_f64(__frcp_rn(f64_to_f32_trunc23(ax)), m, E);
    const double e = fma(-ax, y, 1.0);
    const float ef = signed_trunc23(e);
    const float q = ef * ef * (1.0f + ef);
    const double k = e + f32_to_f64_signed(q);
    return __longlong_as_double(__double_as_longlong(fma(y, k, y)) ^ sgn);
}

// Exact FP64 pair contribution, in the reference's operation order
// (src/common.c:61-70): r = sqrt(r2); r3 = r * r2; a -= (gm*d)/r3.
__device__ __forceinline__ void pair_exact(double xj, double yj, double zj, const Src &s,
                                           double &ax, double &ay, double &az)
{
    double dx = xj - s.x;
    double dy = yj - s.y;
    double dz = zj - s.z;
    double r2 = dx * dx + dy * dy + dz * dz;
    double r1 = sqrt(r2);
    double r3 = r1 * r2;
    ax -= s.gm * dx / r3;
    ay -= s.gm * dy / r3;
    az -= s.gm * dz / r3;
}

// Fast FP64 pair contribution: 6 FP64 instructions (3 separations, 3
// accumulations); r2 and G m r^-3 are integer arithmetic (r2_int,
// gm_inv_r3_int; a C restatement of the whole term over 2 million random
// separations (1e-9 .. 2e4 per component, some zero), masses and seeds
// perturbed by 2^-22: at most 0.53 ulp from the exact G m r^-3, mean
// signed error +0.001 ulp).
__device__ __forceinline__ void pair_fast(double xj, double yj, double zj, const Src &s,
                                          double &ax, double &ay, double &az)
{
    const double dx = xj - s.x;
    const double dy = yj - s.y;
    const double dz = zj - s.z;
    unsigned long long Mr;
    int Er;
    r2_int(dx, dy, dz, Mr, Er);
    const double w = gm_inv_r3_int(Mr, Er, s.gm);
    ax = fma(-w, dx, ax);
    ay = fma(-w, dy, ay);
    az = fma(-w, dz, az);
}

// The plain FP64 GPU pair term of the reference's gpuforce_v2
// (src/gpuforce.cu:61-84, without softening): d2 = dx^2 + dy^2 + dz^2,
// skipped when zero, 1/sqrt by the CUDA rsqrt, inv^3, a -= G m d inv^3.
// Written as plain expressions: the unit that uses it is compiled with FMA
// contraction, as a straightforward port would be.
__device__ __forceinline__ void pair_naive(double xj, double yj, double zj, const Src &s,
                                           double &ax, double &ay, double &az)
{
    const double dx = xj - s.x;
    const double dy = yj - s.y;
    const double dz = zj - s.z;
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (d2 == 0.0) return;
    const double inv = rsqrt(d2);
    const double inv3 = inv * inv * inv;
    ax -= s.gm * dx * inv3;
    ay -= s.gm * dy * inv3;
    az -= s.gm * dz * inv3;
}

// A double as the sum of two floats of 24 significant bits each, by integer
// instructions only: hi is x truncated to 24 bits, lo the rest truncated to
// 24 bits, so |x - (hi + lo)| < 2^-47 |x| and both carry x's sign.  x must
// be zero or have its magnitude within the float range (about 1.2e-38 ..
// 3.4e38); values below it give (0, 0), and a lo part below it is dropped.
__device__ __forceinline__ float2 split_ff(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
    const int ex = (int)((b >> 52) & 0x7FF);
    const int fe = ex - 1023 + 127;
    if (fe < 1) return make_float2(0.0f, 0.0f);
    const unsigned long long M = b & 0xFFFFFFFFFFFFFull;
    const float hi = __uint_as_float(sgn | ((unsigned)min(fe, 254) << 23) | (unsigned)(M >> 29));
    const unsigned r = (unsigned)(M & 0x1FFFFFFFull);  // the 29 bits below hi
    const int lz = __clz(r);                           // 3..32
    const int le = ex - 917 - lz;                      // float exponent of r's leading bit
    const float lo = (r == 0u || le < 1)
                         ? 0.0f
                         : __uint_as_float(sgn | ((unsigned)le << 23) | (((r << lz) >> 8) & 0x7FFFFFu));
    return make_float2(hi, lo);
}

// A float as a double, exactly, by integer instructions (zero and subnormal
// floats give zero; infinities and NaN are not expected).
__device__ __forceinline__ double f32_to_f64_exact(float f)
{
    const unsigned b = __float_as_uint(f);
    if ((b & 0x7F800000u) == 0u) return 0.0;
    const unsigned sgn = b & 0x80000000u;
    const unsigned a = b & 0x7FFFFFFFu;
    return __hiloint2double((int)(((a >> 3) + ((1023 - 127) << 20)) | sgn), (int)(a << 29));
}

// One term w d added to the two-float sum (S, C) in single precision: the
// product of the two-float factors to about 2^-46 (the exact error of
// w_hi d_hi by fmaf, plus the cross terms) and S + p by TwoSum, whose exact
// rounding error goes to C with the product's.  The unit is built without
// FMA contraction, so every other operation rounds as written.
__device__ __forceinline__ void ff_add_product(float2 w, float2 d, float &S, float &C)
{
    const float p = w.x * d.x;
    float pe = fmaf(w.x, d.x, -p);
    pe = fmaf(w.x, d.y, pe);
    pe = fmaf(w.y, d.x, pe);
    const float sm = S + p;
    const float z = sm - S;
    const float t = (S - (sm - z)) + (p - z);
    C = C + (t + pe);
    S = sm;
}

// Two-float (hi + lo) arithmetic in single precision for the mixed forms,
// after Dekker and Knuth: TwoSum and FMA-based TwoProd give the exact
// rounding errors, renormalised by Fast2Sum, about 2^-46 relative.  The
// library is built without FMA contraction, so every step rounds as written.
__device__ __forceinline__ float2 ff_fast_two_sum(float a, float b)
{
    const float s = a + b;
    return make_float2(s, b - (s - a));
}

__device__ __forceinline__ float2 ff_add(float2 a, float2 b)
{
    const float s = a.x + b.x;
    const float z = s - a.x;
    const float e = (a.x - (s - z)) + (b.x - z);
    return ff_fast_two_sum(s, e + (a.y + b.y));
}

__device__ __forceinline__ float2 ff_sub(float2 a, float2 b)
{
    return ff_add(a, make_float2(-b.x, -b.y));
}

__device__ __forceinline__ float2 ff_mul(float2 a, float2 b)
{
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return ff_fast_two_sum(p, e);
}

__device__ __forceinline__ float2 ff_sqr(float2 a)
{
    const float p = a.x * a.x;
    const float e = fmaf(a.x, a.x, -p);
    return ff_fast_two_sum(p, fmaf(2.0f * a.x, a.y, e));
}

// 1/sqrt(x) for a positive two-float x within the float range: the
// rsqrtf seed y and one correction from the expansion
// x^(-1/2) = y (1 - e)^(-1/2) = y (1 + e/2 + 3/8 e^2 + O(e^3)), e = 1 - x y^2
// evaluated in two-float arithmetic (e itself is below 2^-21).
__device__ __forceinline__ float2 ff_rsqrt(float2 x)
{
    const float y = rsqrtf(x.x);
    const float2 t = ff_mul(x, ff_sqr(make_float2(y, 0.0f)));
    const float2 e = ff_sub(make_float2(1.0f, 0.0f), t);
    const float k = e.x * fmaf(0.375f, e.x, 0.5f);
    return ff_fast_two_sum(y, y * k);
}

// Non-negative doubles keep their order when read as unsigned integers, so
// a max over |v| can be an integer atomicMax.  0 encodes "no value seen";
// NaN is skipped, like the reference's vector_max_abs (src/common.c:192-198).
__device__ __forceinline__ unsigned long long absmax_key(double v)
{
    // integer instructions only: |v|'s bits, NaN (above the infinity
    // pattern) -> 0
    const unsigned long long a = (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull;
    return a <= 0x7FF0000000000000ull ? a + 1ull : 0ull;
}

// Finite test on the exponent bits (no FP64 instruction).
__device__ __forceinline__ bool finite_bits(double v)
{
    return ((unsigned)__double2hiint(v) & 0x7FF00000u) != 0x7FF00000u;
}

__host__ __device__ inline double absmax_value(unsigned long long key)
{
#ifdef __CUDA_ARCH__
    return key ? __longlong_as_double((long long)(key - 1ull)) : -1.7976931348623157e308;
#else
    if (!key) return -1.7976931348623157e308;
    unsigned long long b = key - 1ull;
    double d;
    memcpy(&d, &b, sizeof d);
    return d;
#endif
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

}  // namespace abie
