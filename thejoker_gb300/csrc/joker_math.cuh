// Device math for the likelihood kernels: Kepler solvers (FP64 and FP32),
// float-float (double-single) arithmetic, and numpy's PCG64 generator.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "joker_sincos_table.cuh"

namespace joker {

constexpr double PI_D = 3.141592653589793238462643383279502884;
constexpr double TWO_PI_D = 6.283185307179586476925286766559005768;
constexpr double TWO_PI_HI_D = 6.283185307179586;          // nearest double to 2 pi
constexpr double TWO_PI_LO_D = 2.4492935982947064e-16;     // 2 pi - TWO_PI_HI_D
constexpr double INV_TWO_PI_D = 0.15915494309189533577;
constexpr float PI_F = 3.14159265358979f;
constexpr float TWO_PI_HI_F = 6.28318548202514648f;         // nearest float to 2 pi
constexpr float TWO_PI_LO_F = -1.7484556e-07f;              // 2 pi - TWO_PI_HI_F
// Markley (1995) starter: alpha = (3 pi^2 + 1.6 pi (pi - |M|) / (1 + e)) / (pi^2 - 6)
constexpr double MK_A0_D = 3.0 * PI_D * PI_D / (PI_D * PI_D - 6.0);
constexpr double MK_A1_D = 1.6 * PI_D / (PI_D * PI_D - 6.0);

// --------------------------------------------------------- float-float helpers
// Knuth's two-sum: s + err = a + b exactly.  The _rn intrinsics keep the
// compiler from contracting it into FMAs.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &err) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ double ff_to_double(float hi, float lo) {
    return (double)hi + (double)lo;
}

__device__ __forceinline__ float fast_rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// ----------------------------------------------------------------- FP64 Kepler
// This GPU's FP64 throughput is about 1/74 of its FP32 throughput (measured
// FMA rates), so the FP64 solver does in FP64 only what needs FP64 resolution: the
// starter is FP32, sin and cos come from a table plus short Taylor series,
// and the reciprocals from Newton's iteration.

// Reciprocal by Newton-Raphson: the hardware estimate (PTX rcp.approx.ftz.f64)
// refined by two steps r <- r + r (1 - x r), each of which squares the
// relative error.  For the callers' arguments (positive, >= 2^-60) the result
// is within about an ulp of 1/x.
__device__ __forceinline__ double rcp_newton(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    r = fma(r, fma(-x, r, 1.0), r);
    return fma(r, fma(-x, r, 1.0), r);
}

// sin and cos, to FP64 accuracy, of an FP32 angle a in [0, 403.5/128]: with
// k = round(128 a), r = a - k/128 is exact in FP32 and |r| <= 1/256, so
// sin r = r - r^3/6 + r^5/120 and cos r - 1 = -r^2/2 + r^4/24 leave
// truncation errors below 2^-60; the angle-addition formulas combine them
// with the tabulated sin, cos of k/128.  k is clamped to the table, so any
// input (NaN included) reads inside it.
__device__ __forceinline__ void sincos_f32arg(float a, double &s, double &c) {
    int k = __float2int_rn(a * 128.0f);
    k = min(max(k, 0), SINCOS_TAB_N - 1);
    const double r = (double)__fmaf_rn((float)k, -0.0078125f, a);
    const double2 t = __ldg(&kSinCos128[k]);
    const double r2 = r * r;
    const double sr = fma(r * r2, fma(r2, 1.0 / 120.0, -1.0 / 6.0), r);
    const double cm1 = r2 * fma(r2, 1.0 / 24.0, -0.5);
    s = fma(t.x, cm1, fma(t.y, sr, t.x));
    c = fma(t.y, cm1, fma(-t.x, sr, t.y));
}

// Markley's starter (F. L. Markley, 1995, "Kepler equation solver", Celestial
// Mechanics and Dynamical Astronomy 63, 101-111) in FP32 for x = |M| in
// [0, pi]: the root of a cubic model of Kepler's equation, within about 4e-4
// rad of E.  ome = 1 - e and a1 = 1.6 pi / ((1 + e)(pi^2 - 6)) are the
// sample's constants.  The discriminant is clamped at zero (it is >= 0 in
// exact arithmetic), so x = 0 gives E1 = 0.
__device__ __forceinline__ float markley_starter_f32(float x, float e, float ome, float a1) {
    const float alpha = __fmaf_rn(a1, PI_F - x, (float)MK_A0_D);
    const float d = __fmaf_rn(alpha, e, 3.0f * ome);
    const float x2 = x * x;
    const float ad = alpha * d;
    const float q = __fmaf_rn(2.0f * ad, ome, -x2);
    const float r = x * __fmaf_rn(3.0f * ad, d - ome, x2);
    const float sq = sqrtf(fmaxf(__fmaf_rn(q * q, q, r * r), 0.0f));
    const float w = exp2f(0.6666667f * __log2f(r + sq));          // (r + sq)^(2/3)
    const float den3 = __fmaf_rn(w, w + q, q * q);
    return __fmaf_rn(x, den3, 2.0f * r * w) * fast_rcp(den3 * d);
}

// FP64 eccentric anomaly of M in [-pi, pi] for 0 <= e < 1, returned as
// (sin E, cos E).  ef, omef = 1 - e and a1f (markley_starter_f32) are the
// sample's FP32 constants.  From the FP32 starter E1 (exact as a double) and
// its FP64 sin and cos, the root of f(E) = E - e sin E - |M| is E1 + delta,
// delta from the reversion of f's Taylor series about E1 to fourth order in
// u = -f/f': with t2 = f''/f' and t3 = f'''/f' (and f'''' = -f''),
//   delta = u - (t2/2) u^2 + (t2^2/2 - t3/6) u^3
//             + t2 (1/24 + 5 t3/12 - 5 t2^2/8) u^4,
// whose error is of order u^5 (the order of Markley's own fifth-order
// correction); (sin E1, cos E1) are then rotated through delta by its Taylor
// series (|delta| < 5e-4).
__device__ __forceinline__ void kepler_sincos_f64(double M, double e, float ef, float omef,
                                                  float a1f, double &sinE, double &cosE) {
    const double x = fabs(M);
    const float E1f = markley_starter_f32((float)x, ef, omef, a1f);
    double s1, c1;
    sincos_f32arg(E1f, s1, c1);
    const double f2 = e * s1;
    const double f3 = e * c1;
    const double f0 = ((double)E1f - x) - f2;
    const double i1 = rcp_newton(1.0 - f3);
    const double u = -f0 * i1;
    const double t2 = f2 * i1;
    const double t3 = f3 * i1;
    const double t22 = t2 * t2;
    const double c3 = fma(t22, 0.5, t3 * (-1.0 / 6.0));
    const double c4 = t2 * fma(t22, -0.625, fma(t3, 5.0 / 12.0, 1.0 / 24.0));
    const double d = u * fma(u, fma(u, fma(u, c4, c3), -0.5 * t2), 1.0);
    const double dd = d * d;
    const double cm1 = dd * fma(dd, 1.0 / 24.0, -0.5);
    const double sd = d * fma(dd, -1.0 / 6.0, 1.0);
    const double sE = fma(s1, cm1, fma(c1, sd, s1));
    cosE = fma(c1, cm1, fma(-s1, sd, c1));
    sinE = (M < 0.0) ? -sE : sE;
}

// The FP32 constants of kepler_sincos_f64 for eccentricity e.
__device__ __forceinline__ void kepler_consts_f32(double e, float &ef, float &omef, float &a1f) {
    ef = (float)e;
    omef = (float)(1.0 - e);
    a1f = (float)MK_A1_D * fast_rcp(1.0f + ef);
}

// sin and cos of a double angle a to about an ulp (for |a| up to ~1e6 rad;
// NaN in, NaN out): a is reduced to x in [-pi, pi] with the two-part 2 pi,
// |x| = k/128 + r with |r| <= 1/256 (exact by Sterbenz's lemma), and sin r,
// cos r - 1 from the same Taylor series as sincos_f32arg.
__device__ __forceinline__ void sincos_f64_table(double a, double &s, double &c) {
    const double nrev = rint(a * INV_TWO_PI_D);
    double x = fma(-nrev, TWO_PI_HI_D, a);
    x = fma(-nrev, TWO_PI_LO_D, x);
    const double ax = fabs(x);
    int k = __float2int_rn((float)ax * 128.0f);
    k = min(max(k, 0), SINCOS_TAB_N - 1);
    const double r = fma((double)k, -0.0078125, ax);
    const double2 t = __ldg(&kSinCos128[k]);
    const double r2 = r * r;
    const double sr = fma(r * r2, fma(r2, 1.0 / 120.0, -1.0 / 6.0), r);
    const double cm1 = r2 * fma(r2, 1.0 / 24.0, -0.5);
    const double sa = fma(t.x, cm1, fma(t.y, sr, t.x));
    c = fma(t.y, cm1, fma(-t.x, sr, t.y));
    s = (x < 0.0) ? -sa : sa;
}

// x^(-1/3) (other x: the library pow).  For a positive normal x = v 2^(3q), v in [1, 8)
// (integer exponent arithmetic), an FP32 estimate of v^(-1/3) is refined by
// two Newton-Raphson steps on f(y) = y^-3 - v, y <- y (4 - v y^3) / 3, each
// of which squares the relative error (2^-21 -> 2^-41 -> below rounding);
// the result is y 2^-q.
__device__ __forceinline__ double rcbrt_newton(double x) {
    const int hi = __double2hiint(x);
    const int ex = ((hi >> 20) & 0x7ff) - 1023;
    if (hi < 0 || ex == -1023 || ex == 1024) return pow(x, -1.0 / 3.0);   // <= 0, subnormal, inf, NaN
    const int q = (ex + 3072) / 3 - 1024;                 // floor(ex / 3)
    const int rr = ex - 3 * q;                             // 0, 1, 2
    const double v = __hiloint2double((hi & 0x000fffff) | ((rr + 1023) << 20),
                                      __double2loint(x));
    double y = (double)exp2f(-0.33333334f * __log2f((float)v));
    y = y * (fma(-v, y * y * y, 4.0) * (1.0 / 3.0));
    y = y * (fma(-v, y * y * y, 4.0) * (1.0 / 3.0));
    return y * __hiloint2double((1023 - q) << 20, 0);
}

__device__ __forceinline__ void kepler_sincos_f64(double M, double e, double &sinE,
                                                  double &cosE) {
    float ef, omef, a1f;
    kepler_consts_f32(e, ef, omef, a1f);
    kepler_sincos_f64(M, e, ef, omef, a1f, sinE, cosE);
}

// ------------------------------------------------------------------- PCG64
// numpy's PCG64 (128-bit LCG, XSL-RR output; M. E. O'Neill, "PCG: A family of
// simple fast space-efficient statistically good algorithms for random number
// generation", 2014).  Generator.uniform draws one 64-bit output per double:
// u = (x >> 11) * 2^-53.  The state is stepped before each output.
typedef unsigned __int128 u128;
__device__ __forceinline__ u128 pcg_mult() {
    return ((u128)0x2360ED051FC65DA4ull << 64) | (u128)0x4385DF649FCCF645ull;
}

__device__ __forceinline__ u128 pcg_step(u128 s, u128 inc) { return s * pcg_mult() + inc; }

__device__ __forceinline__ uint64_t pcg_output(u128 s) {
    const unsigned rot = (unsigned)(s >> 122);
    const uint64_t x = (uint64_t)(s >> 64) ^ (uint64_t)s;
    return (x >> rot) | (x << ((64u - rot) & 63u));
}

// Advance an LCG by delta steps in O(log delta) (F. B. Brown, 1994, "Random
// number generation with arbitrary strides", Trans. Am. Nucl. Soc. 71, 202).
__device__ __forceinline__ u128 pcg_advance(u128 s, u128 inc, uint64_t delta) {
    u128 cm = pcg_mult(), cp = inc, am = 1, ap = 0;
    while (delta) {
        if (delta & 1) { am *= cm; ap = ap * cm + cp; }
        cp = (cm + 1) * cp;
        cm *= cm;
        delta >>= 1;
    }
    return am * s + ap;
}

// Stepping the LCG n times maps s -> A^n s + S_n inc, S_n = 1 + A + ... + A^(n-1).
// Tables of (A^n, S_n) for n = 2^k and for n = 0..32, computed at compile time:
// (A^2n, S_2n) = (A^n A^n, S_n (1 + A^n)), (A^(l+1), S_(l+1)) = (A A^l, S_l + A^l).
struct PcgTables {
    unsigned long long dbl_a[64][2], dbl_s[64][2];
    unsigned long long lane_a[33][2], lane_s[33][2];
};

constexpr PcgTables make_pcg_tables() {
    PcgTables t{};
    const u128 A = ((u128)0x2360ED051FC65DA4ull << 64) | (u128)0x4385DF649FCCF645ull;
    u128 a = A, sum = 1;
    for (int k = 0; k < 64; ++k) {
        t.dbl_a[k][0] = (unsigned long long)a; t.dbl_a[k][1] = (unsigned long long)(a >> 64);
        t.dbl_s[k][0] = (unsigned long long)sum; t.dbl_s[k][1] = (unsigned long long)(sum >> 64);
        sum = sum * (a + 1);
        a = a * a;
    }
    u128 al = 1, sl = 0;
    for (int l = 0; l <= 32; ++l) {
        t.lane_a[l][0] = (unsigned long long)al; t.lane_a[l][1] = (unsigned long long)(al >> 64);
        t.lane_s[l][0] = (unsigned long long)sl; t.lane_s[l][1] = (unsigned long long)(sl >> 64);
        sl = sl + al;
        al = al * A;
    }
    return t;
}

__constant__ PcgTables g_pcg = make_pcg_tables();

__device__ __forceinline__ u128 u128_of(const unsigned long long (&v)[2]) {
    return ((u128)v[1] << 64) | (u128)v[0];
}

// Advance by n steps with the doubling table (popcount(n) multiply-adds).
__device__ __forceinline__ u128 pcg_jump(u128 s, u128 inc, uint64_t n) {
    for (int k = 0; n; ++k, n >>= 1)
        if (n & 1) s = u128_of(g_pcg.dbl_a[k]) * s + u128_of(g_pcg.dbl_s[k]) * inc;
    return s;
}

__device__ __forceinline__ double pcg_uniform(uint64_t x) {
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

// (A^n, S_n) for n = 1..128 as {A lo, A hi, S lo, S hi}: entry t takes a
// state at position p to the state of position p + t + 1, so that thread t
// of a 128-thread block (or lane t of a warp) draws the uniform of sample
// p + t.  In global memory: a warp reads its 32 entries as one coalesced
// 1 KB line set, where the constant bank would serialise 32 addresses.
struct PcgThreadTable {
    unsigned long long v[128][4];
};

constexpr PcgThreadTable make_pcg_thread_table() {
    PcgThreadTable t{};
    const u128 A = ((u128)0x2360ED051FC65DA4ull << 64) | (u128)0x4385DF649FCCF645ull;
    u128 an = A, sn = 1;                                  // n = 1
    for (int k = 0; k < 128; ++k) {
        t.v[k][0] = (unsigned long long)an; t.v[k][1] = (unsigned long long)(an >> 64);
        t.v[k][2] = (unsigned long long)sn; t.v[k][3] = (unsigned long long)(sn >> 64);
        sn = sn + an;
        an = an * A;
    }
    return t;
}

__device__ PcgThreadTable g_pcg_thr = make_pcg_thread_table();

// (A^n, S_n) for n = 32 w, w = 0..255: from the state of the first sample of
// an 8192-sample block to that of word w (same layout).
struct PcgWordTable {
    unsigned long long v[256][4];
};

constexpr PcgWordTable make_pcg_word_table() {
    PcgWordTable t{};
    const u128 A = ((u128)0x2360ED051FC65DA4ull << 64) | (u128)0x4385DF649FCCF645ull;
    u128 a32 = 1, s32 = 0;                                // (A^32, S_32)
    for (int k = 0; k < 32; ++k) { s32 = s32 + a32; a32 = a32 * A; }
    u128 an = 1, sn = 0;                                  // n = 0
    for (int w = 0; w < 256; ++w) {
        t.v[w][0] = (unsigned long long)an; t.v[w][1] = (unsigned long long)(an >> 64);
        t.v[w][2] = (unsigned long long)sn; t.v[w][3] = (unsigned long long)(sn >> 64);
        sn = sn * a32 + s32;                              // S_(n+32) = S_n A^32 + S_32
        an = an * a32;
    }
    return t;
}

__device__ PcgWordTable g_pcg_w32 = make_pcg_word_table();

// State of position p + t + 1 from the state x of position p.
__device__ __forceinline__ u128 pcg_thread_step(u128 x, u128 inc, int t) {
    const unsigned long long *e = g_pcg_thr.v[t];
    return (((u128)e[1] << 64) | (u128)e[0]) * x + (((u128)e[3] << 64) | (u128)e[2]) * inc;
}

// u = m 2^-53 (m the 53-bit integer of numpy's uniform double) as a float
// truncated to 24 significant bits; m must be nonzero.
__device__ __forceinline__ float u53_to_float(uint64_t m) {
    const int lz = __clzll(m);                       // 11..63
    const uint64_t norm = m << lz;                   // leading one at bit 63
    const unsigned mant = (unsigned)(norm >> 40) & 0x7fffffu;
    const int e2 = 63 - lz - 53;                     // u in [2^e2, 2^(e2+1))
    return __int_as_float(((e2 + 127) << 23) | (int)mant);
}

}  // namespace joker

namespace joker {

// ------------------------------------------------------ float-float numbers
// A value hi + lo with |lo| <= ulp(hi)/2 after normalisation: a 48-bit
// significand with FP32 exponent range (Dekker 1971; Hida, Li and Bailey,
// "Library for double-double and quad-double arithmetic", 2001).
struct ff {
    float hi, lo;
};

__device__ __forceinline__ ff ff_make(float hi, float lo) { ff r; r.hi = hi; r.lo = lo; return r; }

// requires |a| >= |b| or a == 0
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return ff_make(s, __fsub_rn(b, __fsub_rn(s, a)));
}

__device__ __forceinline__ ff ff_norm(float hi, float lo) {
    float s, e;
    two_sum(hi, lo, s, e);
    return ff_make(s, e);
}

__device__ __forceinline__ ff ff_addf(ff a, ff b) {
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    return fast_two_sum(s, e);
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff_make(-a.hi, -a.lo); }

__device__ __forceinline__ ff ff_subf(ff a, ff b) { return ff_addf(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mulf(ff a, ff b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ ff ff_mul1(ff a, float b) {
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ ff ff_divf(ff a, ff b) {
    const float r = __frcp_rn(b.hi);
    const float q1 = __fmul_rn(a.hi, r);
    const ff rem = ff_subf(a, ff_mul1(b, q1));
    const float q2 = __fmul_rn(rem.hi, r);
    return fast_two_sum(q1, q2);
}

__device__ __forceinline__ double ff_to_d(ff a) { return (double)a.hi + (double)a.lo; }

// Natural log of a positive float-float number to about 1e-7 absolute: the
// binary exponent is exact, the mantissa goes through logf, the low word
// through log(1 + x) ~ x.
__device__ __forceinline__ float ff_log(ff a) {
    const int bits = __float_as_int(a.hi);
    const int ex = ((bits >> 23) & 0xff) - 127;
    const float m = __int_as_float((bits & 0x807fffff) | 0x3f800000);   // [1, 2)
    return (float)ex * 0.69314718f + logf(m) + a.lo / a.hi;
}

// ---- per-sample preparation of the mixed path -----------------------------
// Split a double into an unevaluated float pair: hi = x with its mantissa
// truncated to 24 bits, lo = the remaining 29 bits rounded to a float, so
// |hi + lo - x| <= 2^-48 |x|.  Integer operations only (GB300's FP64 and
// FP64-conversion rate is 1/64 of FP32).  Zero, values outside the float
// normal range, inf and NaN go through one FP64 conversion with lo = 0.
__device__ __forceinline__ void split_d2ff(double x, float &hi, float &lo) {
    const long long b = __double_as_longlong(x);
    if ((b & 0x7fffffffffffffffLL) == 0) { hi = 0.0f; lo = 0.0f; return; }
    const int hw = (int)(b >> 32);
    const int ex = (hw >> 20) & 0x7ff;
    if (ex < 897 || ex > 1150) { hi = __double2float_rn(x); lo = 0.0f; return; }
    const unsigned sign = (unsigned)hw & 0x80000000u;
    hi = __uint_as_float(sign | ((unsigned)(ex - 896) << 23) | ((unsigned)(b >> 29) & 0x7fffffu));
    const unsigned rem = (unsigned)b & 0x1fffffffu;           // the 29 bits below hi
    const float scale = ex >= 949 ? __uint_as_float((unsigned)(ex - 948) << 23) : 0.0f;
    lo = __uint_as_float(sign | __float_as_uint(__uint2float_rn(rem) * scale));
}

// 1/(2 pi) and 1/pi as float pairs (hi = the float nearest, lo = the rest).
constexpr float INV_2PI_HI_F = 0x1.45f306p-3f, INV_2PI_LO_F = 0x1.b93910p-28f;
constexpr float INV_PI_HI_F = 0x1.45f306p-2f, INV_PI_LO_F = 0x1.b93910p-27f;

// Product of a float pair with a constant float pair, as a float pair.
__device__ __forceinline__ void mul_ff_const(float xh, float xl, float ch, float cl, float &ph,
                                             float &pl) {
    ph = __fmul_rn(xh, ch);
    float pe = __fmaf_rn(xh, ch, -ph);
    pe = __fmaf_rn(xh, cl, pe);
    pl = __fmaf_rn(xl, ch, pe);
}

// The prepared form of one prior sample (P, e, omega, M0, s) read by the
// mixed kernel:
//   a = (1/P hi, 1/P lo, M0/2pi mod 1 hi, lo)    float pairs, ~2^-46 relative
//   b = (e, cos omega, sin omega, log g),  g = P^(-2/3) / (1 - e^2)
//   s2 = s^2
// FP32 and integer arithmetic only.  The cache preparation and the kernel
// that reads packed FP64 rows directly both use it, so they agree bit for bit.
__device__ __forceinline__ void prepare_sample(double p, double e, double om, double m0, double s,
                                               float4 &pa, float4 &pb, float &s2) {
    float ph, pl;
    split_d2ff(p, ph, pl);
    // 1/P: the float reciprocal of hi, corrected once with the exact residual
    const float r0 = __frcp_rn(ph);
    float t = __fmaf_rn(-ph, r0, 1.0f);
    t = __fmaf_rn(-pl, r0, t);
    const float r1 = __fmul_rn(r0, t);
    const float ip_hi = __fadd_rn(r0, r1);
    const float ip_lo = __fadd_rn(__fsub_rn(r0, ip_hi), r1);
    // M0 / 2 pi, reduced to [0, 1) (c - floor(c) is exact)
    float mh, ml, c, ce;
    split_d2ff(m0, mh, ml);
    mul_ff_const(mh, ml, INV_2PI_HI_F, INV_2PI_LO_F, c, ce);
    c = __fsub_rn(c, floorf(c));
    float mc_hi, mc_lo;
    two_sum(c, ce, mc_hi, mc_lo);
    // omega / pi, reduced to [0, 2), then sin and cos of pi times it
    float oh, ol, w, we;
    split_d2ff(om, oh, ol);
    mul_ff_const(oh, ol, INV_PI_HI_F, INV_PI_LO_F, w, we);
    w = __fsub_rn(w, 2.0f * floorf(0.5f * w));
    float sw, cw;
    sincospif(__fadd_rn(w, we), &sw, &cw);
    // e and e^2 (to one rounding), log g
    float eh, el;
    split_d2ff(e, eh, el);
    const float ef = __fadd_rn(eh, el);
    const float e2h = __fmul_rn(eh, eh);
    const float e2 = __fadd_rn(e2h, __fmaf_rn(eh, eh, -e2h) + 2.0f * eh * el);
    const float lg = -0.6666667f * logf(__fadd_rn(ph, pl)) - log1pf(-e2);
    float sh, sl;
    split_d2ff(s, sh, sl);
    const float s2h = __fmul_rn(sh, sh);
    s2 = __fadd_rn(s2h, __fmaf_rn(sh, sh, -s2h) + 2.0f * sh * sl);
    pa = make_float4(ip_hi, ip_lo, mc_hi, mc_lo);
    pb = make_float4(ef, cw, sw, lg);
}

}  // namespace joker
