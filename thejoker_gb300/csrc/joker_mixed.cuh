// The mixed-precision ln L kernel (FP32 Kepler, float-float epoch sums,
// per-sample error bound) and the helpers the ln L kernels share.  A header
// so that its two forms -- reading the prepared cache, or reading packed
// FP64 rows and preparing each sample in registers -- compile in separate
// translation units.
#pragma once
#include "joker_fp64.cuh"

namespace joker {

// ------------------------------------------------------------------ staging
template <typename T, int REC>
__device__ __forceinline__ void stage_epochs(T *sm, const T *src, int n) {
    const int nvec = n * REC * (int)sizeof(T) / 16;
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
    float4 *d4 = reinterpret_cast<float4 *>(sm);
    for (int i = threadIdx.x; i < nvec; i += blockDim.x) d4[i] = __ldg(s4 + i);
}

// Warp-aggregated raise of a running maximum.
__device__ __forceinline__ void warp_max_update(unsigned long long *key, unsigned long long k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, k, o);
        k = other > k ? other : k;
    }
    if ((threadIdx.x & 31) == 0 && k != 0ull) {
        if (k > *((volatile unsigned long long *)key)) atomicMax(key, k);
    }
}

// ----------------------------------------------------------- K2: mixed path
// Epoch record (REC32 floats), no jitter:
//   dt_hi, dt_lo, w_hi, w_lo, wy_hi, wy_lo, (wT_j hi, lo) j = 1..L-1
// with jitter:
//   dt_hi, dt_lo, ivar, 0, y_hi, y_lo, ysq_hi, ysq_lo, (T_j hi, lo) j = 1..L-1
// VAR: 0 = MUFU sin/cos + float-float tail, 1 = correctly rounded sincosf +
// float-float tail, 2 = MUFU sin/cos + FP64 tail.
//
// Error bound per sample.  The FP32 column m carries an error |dm| <= D with
// D = c0 (1 + e) / (1 - e)^2 (phase rounding and FP32 Kepler, amplified near
// pericentre of eccentric orbits); all epoch sums are exact functions of the
// FP32 column.  To first order chi2 changes by -2 K_hat sum w res dm and
// s by 2 sum w m_perp dm, so with W = sum ivar
//   |d chi2| <= 2 |K_hat| D sqrt(W chi2) + K_hat^2 D^2 W
//   |d s|    <= 2 D sqrt(W (s - 1/Lambda0)) + W D^2
// and |d lnL| <= (|d chi2| + |d s| / (s - |d s|)) / 2 plus rounding terms.
// With the jitter applied each weight w = ivar / (1 + s^2 ivar) is an FP32
// value (relative error ~2^-22); the sums use it consistently, so chi2 moves
// by sum dw res^2 <= 2e-7 chi2 and sum log w by the FP32 log2 error per epoch.
//
// PACKED: read each sample as FP64 (P, e, omega, M0, s) from a.P.. with
// stride a.stride (the reference's packed chunk, in device memory or mapped
// pinned host memory) and prepare it in registers (prepare_sample), instead of
// reading the prepared cache; the values are identical.
// ---- scalar and paired FP32 arithmetic ------------------------------------
// The epoch loop is written once over T = float (one sample per thread) or
// T = float2 (two samples per thread).  Every operation rounds to nearest
// with no contraction; on float2 the additions, multiplications and FMAs are
// the paired FP32 instructions of sm_100+ (one issue for both samples), and
// the special functions and roundings go lane by lane.  Every step rounds
// like its scalar counterpart; the two forms agree to FP32 rounding (the
// compiler may schedule the lane-wise special functions and the scalar tail
// differently), and each carries its own error bound.
__device__ __forceinline__ float vadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float vsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float vmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ float vneg(float a) { return -a; }
// The paired operations go through inline PTX with an explicit .rn: the
// compiler's f32x2 builtins may be contracted (a product fused into a
// following sum), which would break the error-free two-sum and two-product.
__device__ __forceinline__ unsigned long long f2_bits(float2 a) {
    unsigned long long r;
    memcpy(&r, &a, 8);
    return r;
}
__device__ __forceinline__ float2 bits_f2(unsigned long long r) {
    float2 a;
    memcpy(&a, &r, 8);
    return a;
}
__device__ __forceinline__ float2 vadd(float2 a, float2 b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
    return bits_f2(d);
}
__device__ __forceinline__ float2 vsub(float2 a, float2 b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
    return bits_f2(d);
}
__device__ __forceinline__ float2 vmul(float2 a, float2 b) {
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
    return bits_f2(d);
}
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)), "l"(f2_bits(c)));
    return bits_f2(d);
}
__device__ __forceinline__ float2 vneg(float2 a) { return make_float2(-a.x, -a.y); }

template <class T> __device__ __forceinline__ T vsplat(float x);
template <> __device__ __forceinline__ float vsplat<float>(float x) { return x; }
template <> __device__ __forceinline__ float2 vsplat<float2>(float x) { return make_float2(x, x); }

// Special-function approximations as single explicit instructions, so that
// no surrounding multiply or add can be fused into them differently in the
// two forms.
__device__ __forceinline__ float lg2_approx(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float ex2_approx(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsqrt_approx(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// lane by lane
template <class Fn> __device__ __forceinline__ float vmap(Fn f, float x) { return f(x); }
template <class Fn> __device__ __forceinline__ float2 vmap(Fn f, float2 x) {
    return make_float2(f(x.x), f(x.y));
}
template <class Fn> __device__ __forceinline__ float vmap2(Fn f, float x, float y) { return f(x, y); }
template <class Fn> __device__ __forceinline__ float2 vmap2(Fn f, float2 x, float2 y) {
    return make_float2(f(x.x, y.x), f(x.y, y.y));
}

// -(a b) given the rounded product p = a b and nb = -b: free for a float (a
// negated operand), one paired multiply for a float2
__device__ __forceinline__ float vnegprod(float, float, float p) { return -p; }
__device__ __forceinline__ float2 vnegprod(float2 a, float2 nb, float2) { return vmul(a, nb); }

// error-free transformations on T
template <class T> __device__ __forceinline__ void vtwo_sum(T a, T b, T &s, T &err) {
    s = vadd(a, b);
    const T bb = vsub(s, a);
    err = vadd(vsub(a, vsub(s, bb)), vsub(b, bb));
}
// (hi, lo) += p + pe with the high part exact
template <class T> __device__ __forceinline__ void vff_add(T &hi, T &lo, T p, T pe) {
    T s, e;
    vtwo_sum(hi, p, s, e);
    hi = s;
    lo = vadd(lo, vadd(e, pe));
}
// (hi, lo) += (c_hi + c_lo) * m, the product c_hi * m exact
template <class T> __device__ __forceinline__ void vff_acc(T &hi, T &lo, T c_hi, T c_lo, T m) {
    const T p = vmul(c_hi, m);
    T pe = vfma(c_hi, m, vneg(p));
    pe = vfma(c_lo, m, pe);
    vff_add(hi, lo, p, pe);
}
// x (hi, lo) * (yh, yl) to first order, the product of the highs exact
template <class T> __device__ __forceinline__ void vff_mul(T xh, T xl, T yh, T yl, T &p, T &pe) {
    p = vmul(xh, yh);
    pe = vfma(xh, yh, vneg(p));
    pe = vfma(xh, yl, vfma(xl, yh, pe));
}

// Round to the nearest integer, ties to even.  SHIFT: on the FMA and integer
// pipes instead of the FRND instruction (which shares the special-function
// unit): adding 1.5 2^23 (with v's sign) rounds v at the units digit, and
// taking the shift back off is exact.  For |v| < 2^22 the result is
// rintf(v); beyond, it is an integer whose difference from v is exact (v is
// then a multiple of 1/2 or an integer).  Measured on GB300: 0.3-0.5 % faster
// for the FP32-sum kernel with the jitter applied, whose special-function
// unit is the busier pipe, and 2 % slower without it.
template <bool SHIFT, class T> __device__ __forceinline__ T vrint(T v) {
    if constexpr (SHIFT) {
        const T sh = vmap([](float x) { return copysignf(12582912.0f, x); }, v);
        return vsub(vadd(v, sh), sh);
    } else {
        return vmap([](float x) { return rintf(x); }, v);
    }
}

// FP32 Kepler on T: Markley's starter (markley_starter_f32's cubic, with the
// approximate special functions) and one Halley step; the starter's error
// (< 4e-4 rad) leaves a Halley residual far below FP32 resolution.  M in
// [-pi, pi]; a1 = 1.6 pi / ((1 + e)(pi^2 - 6)) is a per-sample constant.
template <bool ACCURATE, class T>
__device__ __forceinline__ void vkepler(T M, T e, T ne, T ome, T ome3, T a1, T &sinE, T &cosE) {
    const T x = vmap([](float v) { return fabsf(v); }, M);
    const T alpha = vfma(a1, vsub(vsplat<T>(PI_F), x), vsplat<T>((float)MK_A0_D));
    const T d = vfma(alpha, e, ome3);
    const T x2 = vmul(x, x);
    const T ad = vmul(alpha, d);
    const T q = vfma(vadd(ad, ad), ome, vneg(x2));
    const T r = vmul(x, vfma(vmul(vsplat<T>(3.0f), ad), vsub(d, ome), x2));
    const T qq = vmul(q, q);
    const T disc = vfma(qq, q, vmul(r, r));
    const T sq = vmul(disc, vmap([](float v) { return rsqrt_approx(v); }, disc));
    // w = (|r| + sq)^(2/3)
    const T w = vmap([](float v) { return ex2_approx(__fmul_rn(0.6666667f, lg2_approx(v))); },
                     vadd(vmap([](float v) { return fabsf(v); }, r), sq));
    const T den3 = vfma(w, vadd(w, q), qq);
    const T E1 = vmul(vfma(x, den3, vmul(vadd(r, r), w)),
                      vmap([](float v) { return fast_rcp(v); }, vmul(den3, d)));
    T s1, c1;
    if constexpr (sizeof(T) == 4) {
        if (ACCURATE) sincosf(E1, &s1, &c1);
        else __sincosf(E1, &s1, &c1);
    } else {
        if (ACCURATE) { sincosf(E1.x, &s1.x, &c1.x); sincosf(E1.y, &s1.y, &c1.y); }
        else { __sincosf(E1.x, &s1.x, &c1.x); __sincosf(E1.y, &s1.y, &c1.y); }
    }
    const T es = vmul(e, s1);
    const T f0 = vsub(vsub(E1, x), es);
    const T f1 = vfma(ne, c1, vsplat<T>(1.0f));
    // Halley: delta = -f0 f1 / (f1^2 - f0 f2 / 2); nd = -delta
    const T nd = vmul(vmul(f0, f1), vmap([](float v) { return fast_rcp(v); },
                                         vfma(f1, f1, vmul(vmul(vsplat<T>(-0.5f), f0), es))));
    const T nhd2 = vmul(vmul(vsplat<T>(-0.5f), nd), nd);
    const T sE = vfma(vneg(nd), c1, vfma(nhd2, s1, s1));
    cosE = vfma(nd, s1, vfma(nhd2, c1, c1));
    sinE = vmap2([](float m_, float s_) { return m_ < 0.0f ? -s_ : s_; }, M, sE);
}

// Per-sample constants of the epoch loop.
template <class T> struct MixC {
    T iph, ipl, niph, mch, mcl;   // 1/P (float pair), -1/P hi, M0/2pi mod 1 (pair)
    T e, ne, ome, ome3, a1;       // e, -e, 1 - e, 3 (1 - e), Markley's a1
    T Ac, Bc, nDc, Dc;            // unit-K velocity: (Ac cE + Bc sE - Dc) / (1 - e cE) + Dc
    T s2, ns2;                    // s^2, -s^2
    T ih, il;                     // 1/P as ih (12 significant bits) + il (the rest, a float)
};

__device__ __forceinline__ MixC<float> mix_consts(float4 pa, float4 pb, float s2) {
    MixC<float> c;
    c.iph = pa.x; c.ipl = pa.y; c.niph = -pa.x; c.mch = pa.z; c.mcl = pa.w;
    c.ih = __int_as_float(__float_as_int(pa.x) & (int)0xFFFFF000);   // low 12 mantissa bits cleared
    c.il = __fadd_rn(__fsub_rn(pa.x, c.ih), pa.y);                   // pa.x - ih is exact
    const float e = pb.x, ome = 1.0f - e;
    c.e = e; c.ne = -e; c.ome = ome; c.ome3 = 3.0f * ome;
    c.a1 = (float)MK_A1_D * fast_rcp(1.0f + e);
    const float sq1me2 = sqrtf(ome * (1.0f + e));
    c.Ac = pb.y; c.Bc = -pb.z * sq1me2; c.Dc = e * pb.y; c.nDc = -c.Dc;
    c.s2 = s2; c.ns2 = -s2;
    return c;
}

__device__ __forceinline__ MixC<float2> mix_pair(const MixC<float> &u, const MixC<float> &v) {
    MixC<float2> c;
#define JOKER_PAIR(f) c.f = make_float2(u.f, v.f);
    JOKER_PAIR(iph) JOKER_PAIR(ipl) JOKER_PAIR(niph) JOKER_PAIR(mch) JOKER_PAIR(mcl)
    JOKER_PAIR(e) JOKER_PAIR(ne) JOKER_PAIR(ome) JOKER_PAIR(ome3) JOKER_PAIR(a1)
    JOKER_PAIR(Ac) JOKER_PAIR(Bc) JOKER_PAIR(nDc) JOKER_PAIR(Dc) JOKER_PAIR(s2) JOKER_PAIR(ns2)
    JOKER_PAIR(ih) JOKER_PAIR(il)
#undef JOKER_PAIR
    return c;
}

// Epoch sums of one sample (T = float) or two (T = float2).
template <int L, bool JIT, class T> struct Acc32 {
    // no jitter: A00 = sum w m^2, b0 = sum w m y', A0j = sum w m T_j
    T A00h, A00l, bh, bl, Ah[MAXL], Al[MAXL];
    // jitter: sum w m^2, sum w r m, sum w m T_j, sum w T_j T_k, sum w r T_j,
    // sum w r^2, sum log2(1 + s^2 ivar)
    T GKKh, GKKl, qKh, qKl, rh, rl, lg2;
    T GKh[MAXL], GKl[MAXL], GTh[MAXL][MAXL], GTl[MAXL][MAXL], qTh[MAXL], qTl[MAXL];

    __device__ __forceinline__ void zero() {
        const T z = vsplat<T>(0.0f);
        A00h = A00l = bh = bl = z;
        GKKh = GKKl = qKh = qKl = rh = rl = lg2 = z;
#pragma unroll
        for (int i = 0; i < MAXL; ++i) {
            Ah[i] = Al[i] = GKh[i] = GKl[i] = qTh[i] = qTl[i] = z;
#pragma unroll
            for (int k = 0; k < MAXL; ++k) GTh[i][k] = GTl[i][k] = z;
        }
    }
};

// The unit-K RV column m = cos(omega + f) + e cos(omega) at one epoch: the
// phase in cycles dt (1/P) - M0/(2 pi) mod 1 from float pairs (dth, dtl is
// the epoch's dt pair), FP32 Kepler, and the true-anomaly form of the
// velocity.  Shared by the float-float and the FP32-sum kernels.
template <bool ACCURATE, class T>
__device__ __forceinline__ T unit_rv_column(T dth, T dtl, const MixC<T> &c) {
    const T p = vmul(dth, c.iph);
    T pe = vfma(dth, c.iph, vnegprod(dth, c.niph, p));
    pe = vfma(dth, c.ipl, pe);
    pe = vfma(dtl, c.iph, pe);
    const T fr = vsub(p, vrint<false>(p));                                // exact
    T s1, e1;
    vtwo_sum(fr, vneg(c.mch), s1, e1);                                    // exact
    const T lo = vsub(vadd(pe, e1), c.mcl);
    const T k = vrint<false>(vadd(s1, lo));
    const T f = vadd(vsub(s1, k), lo);                                    // [-0.5, 0.5]
    const T M = vfma(f, vsplat<T>(TWO_PI_HI_F), vmul(f, vsplat<T>(TWO_PI_LO_F)));
    T sE, cE;
    vkepler<ACCURATE>(M, c.e, c.ne, c.ome, c.ome3, c.a1, sE, cE);
    const T one = vsplat<T>(1.0f), two = vsplat<T>(2.0f);
    const T den = vfma(c.ne, cE, one);
    const T rd0 = vmap([](float v) { return fast_rcp(v); }, den);
    const T rd = vmul(rd0, vfma(vneg(den), rd0, two));
    return vfma(vfma(c.Ac, cE, vfma(c.Bc, sE, c.nDc)), rd, c.Dc);
}

// One epoch.  recf: the epoch's REC32 float record (the same for every sample
// of the thread; a field is splat into both lanes of a pair).
template <int L, bool JIT, bool ACCURATE, class T>
__device__ __forceinline__ void mixed_epoch(const float *recf, const MixC<T> &c, bool mu0z, T mu0,
                                            T nmu0, Acc32<L, JIT, T> &A) {
    T rec[REC32];
#pragma unroll
    for (int q = 0; q < 8 + 2 * (L - 1); ++q) rec[q] = vsplat<T>(recf[q]);
    const T one = vsplat<T>(1.0f), two = vsplat<T>(2.0f);
    const T m = unit_rv_column<ACCURATE>(rec[0], rec[1], c);
    if constexpr (!JIT) {
        T th, tl;                                                         // w m, exact pair
        th = vmul(rec[2], m);
        tl = vfma(rec[2], m, vneg(th));
        tl = vfma(rec[3], m, tl);
        vff_acc(A.A00h, A.A00l, th, tl, m);
        vff_acc(A.bh, A.bl, rec[4], rec[5], m);
        if (L > 1) vff_add(A.Ah[1], A.Al[1], th, tl);                      // T_1 = 1
#pragma unroll
        for (int kk = 2; kk < L; ++kk) vff_acc(A.Ah[kk], A.Al[kk], rec[4 + 2 * kk], rec[5 + 2 * kk], m);
    } else {
        const T iv = rec[2];
        const T onep = vfma(c.s2, iv, one);
        const T ro0 = vmap([](float v) { return fast_rcp(v); }, onep);
        const T ro = vmul(ro0, vfma(vfma(c.ns2, iv, vsplat<T>(-1.0f)), ro0, two));
        const T wj = vmul(iv, ro);                    // the weight, used consistently
        A.lg2 = vadd(A.lg2, vmap([](float v) { return lg2_approx(v); }, onep));
        // r = y' - mu0 m (float-float)
        T rrh = rec[4], rrl = rec[5];
        if (!mu0z) {
            const T ph = vmul(nmu0, m);
            const T pl = vfma(nmu0, m, vnegprod(m, mu0, ph));
            T s_, e_;
            vtwo_sum(rrh, ph, s_, e_);
            rrl = vadd(vadd(rrl, e_), pl);
            rrh = s_;
        }
        T wmh, wml, wrh, wrl;                          // w m, w r: exact products
        wmh = vmul(wj, m);
        wml = vfma(wj, m, vneg(wmh));
        wrh = vmul(wj, rrh);
        wrl = vfma(wj, rrh, vneg(wrh));
        wrl = vfma(wj, rrl, wrl);
        vff_acc(A.GKKh, A.GKKl, wmh, wml, m);
        vff_acc(A.qKh, A.qKl, wrh, wrl, m);
        if (L > 1) {                                   // T_1 = 1
            vff_add(A.GKh[1], A.GKl[1], wmh, wml);
            T t_, tl_;
            vtwo_sum(A.GTh[1][1], wj, t_, tl_);
            A.GTh[1][1] = t_;
            A.GTl[1][1] = vadd(A.GTl[1][1], tl_);
            vff_add(A.qTh[1], A.qTl[1], wrh, wrl);
        }
        if (mu0z) {                                    // r^2 = y'^2, stored
            const T p1 = vmul(wj, rec[6]);
            T pe1 = vfma(wj, rec[6], vneg(p1));
            pe1 = vfma(wj, rec[7], pe1);
            vff_add(A.rh, A.rl, p1, pe1);
        } else {
            T p1, pe1;
            vff_mul(wrh, wrl, rrh, rrl, p1, pe1);
            vff_add(A.rh, A.rl, p1, pe1);
        }
#pragma unroll
        for (int ii = 2; ii < L; ++ii) {
            const T Th = rec[6 + 2 * ii], Tl = rec[7 + 2 * ii];
            T p2, pe2;
            vff_mul(wmh, wml, Th, Tl, p2, pe2);
            vff_add(A.GKh[ii], A.GKl[ii], p2, pe2);
            vff_mul(wrh, wrl, Th, Tl, p2, pe2);
            vff_add(A.qTh[ii], A.qTl[ii], p2, pe2);
            T wth, wtl;                                // w T_ii
            wth = vmul(wj, Th);
            wtl = vfma(wj, Th, vneg(wth));
            wtl = vfma(wj, Tl, wtl);
            vff_add(A.GTh[ii][1], A.GTl[ii][1], wth, wtl);
#pragma unroll
            for (int kk = 2; kk <= ii; ++kk) {
                vff_mul(wth, wtl, rec[6 + 2 * kk], rec[7 + 2 * kk], p2, pe2);
                vff_add(A.GTh[ii][kk], A.GTl[ii][kk], p2, pe2);
            }
        }
    }
}

// The per-sample tail: the linear solve, ln L and its error bound.
template <int L, bool JIT, int VAR>
__device__ __forceinline__ void mixed_tail(const StarRec &st, const Acc32<L, JIT, float> &A,
                                           float e, float ome, float lgP, int N, float err_c0,
                                           double &lnl, float &err) {
    const bool mu0z = st.mu0_zero != 0;
    const float mu0f = st.mu0_f;
    // K prior variance: log Lambda0 from the per-sample log g
    float log_lam0f;
    if (st.k_scaled) log_lam0f = fminf((float)st.log_maxK2, (float)st.log_kscale + lgP);
    else log_lam0f = (float)log(st.lam0);
    const float ilam0 = expf(-log_lam0f);
    float chi2f = 0.f, s_f = 1.f, amin_f = 0.f, Khat = 0.f, quadf = 0.f;
    err = 0.0f;
    if (VAR == 2) {
        // FP64 tail (the literal FP64 form, kept for comparison)
        const double lam0 = st.k_scaled ? (double)expf(log_lam0f) : st.lam0;
        if (!JIT) {
            double A0d[MAXL];
#pragma unroll
            for (int kk = 0; kk < MAXL; ++kk) A0d[kk] = ff_to_double(A.Ah[kk], A.Al[kk]);
            lnl = tail_schur_d<L, true>(st, ff_to_double(A.A00h, A.A00l), A0d,
                                        ff_to_double(A.bh, A.bl), lam0, (double)log_lam0f);
        } else {
            double G[L][L], q[L];
            G[0][0] = ff_to_double(A.GKKh, A.GKKl) + 1.0 / lam0;
            q[0] = ff_to_double(A.qKh, A.qKl);
#pragma unroll
            for (int ii = 1; ii < L; ++ii) {
                G[ii][0] = G[0][ii] = ff_to_double(A.GKh[ii], A.GKl[ii]);
                q[ii] = ff_to_double(A.qTh[ii], A.qTl[ii]);
#pragma unroll
                for (int kk = 1; kk <= ii; ++kk)
                    G[ii][kk] = G[kk][ii] = ff_to_double(A.GTh[ii][kk], A.GTl[ii][kk]);
                G[ii][ii] += 1.0 / st.lam[ii];
            }
            const double slw = st.sum_log_ivar - 0.6931471805599453 * (double)A.lg2;
            lnl = tail_full_d<L, true>(G, q, ff_to_double(A.rh, A.rl),
                                       st.log_norm_rest + (double)log_lam0f - slw);
        }
        err = 1e30f;   // this variant states no per-sample bound
        return;
    }
    if (!JIT) {
        // float-float Schur-complement tail
        const ff A00 = ff_norm(A.A00h, A.A00l);
        const ff b0 = ff_norm(A.bh, A.bl);
        ff gv = ff_make(0.f, 0.f), gcC = ff_make(0.f, 0.f);
#pragma unroll
        for (int jj = 1; jj < L; ++jj) {
            const ff gj = ff_norm(A.Ah[jj], A.Al[jj]);
            ff vj = ff_make(0.f, 0.f);
#pragma unroll
            for (int kk = 1; kk < L; ++kk)
                vj = ff_addf(vj, ff_mulf(ff_make(st.Cinv_hi[jj * MAXL + kk], st.Cinv_lo[jj * MAXL + kk]),
                                         ff_norm(A.Ah[kk], A.Al[kk])));
            gv = ff_addf(gv, ff_mulf(gj, vj));
            gcC = ff_addf(gcC, ff_mulf(gj, ff_make(st.cC_hi[jj], st.cC_lo[jj])));
        }
        const ff amin = ff_subf(A00, gv);                    // s - 1/Lambda0
        const ff s = ff_addf(amin, ff_make(ilam0, 0.f));
        const ff u = ff_subf(b0, gcC);
        ff t = u;
        ff chi2 = ff_make(st.chi2_0_hi, st.chi2_0_lo);
        if (!mu0z) {
            t = ff_subf(u, ff_mul1(amin, mu0f));
            chi2 = ff_addf(chi2, ff_mul1(ff_subf(ff_mul1(amin, mu0f), ff_mul1(u, 2.0f)), mu0f));
        }
        chi2 = ff_subf(chi2, ff_divf(ff_mulf(t, t), s));
        const float logs = ff_log(s);
        lnl = -0.5 * (ff_to_d(chi2) + st.logdet_const + (double)log_lam0f + (double)logs);
        chi2f = chi2.hi;
        s_f = s.hi;
        amin_f = amin.hi;
        Khat = t.hi / s.hi;
        quadf = Khat * Khat * s_f;
    } else {
        // float-float LDL^T, trend block 1..L-1 first, K last
        ff Dd[MAXL], Lw[MAXL][MAXL], lK[MAXL], z[MAXL];
        float logdet_G = 0.f;
#pragma unroll
        for (int k = 1; k < L; ++k) {
            ff dk = ff_addf(ff_norm(A.GTh[k][k], A.GTl[k][k]), ff_make(st.ilam_hi[k], st.ilam_lo[k]));
#pragma unroll
            for (int mm = 1; mm < k; ++mm) dk = ff_subf(dk, ff_mulf(ff_mulf(Lw[k][mm], Lw[k][mm]), Dd[mm]));
            Dd[k] = dk;
#pragma unroll
            for (int i = k + 1; i < L; ++i) {
                ff v = ff_norm(A.GTh[i][k], A.GTl[i][k]);
#pragma unroll
                for (int mm = 1; mm < k; ++mm) v = ff_subf(v, ff_mulf(ff_mulf(Lw[i][mm], Lw[k][mm]), Dd[mm]));
                Lw[i][k] = ff_divf(v, dk);
            }
            ff v = ff_norm(A.GKh[k], A.GKl[k]);
#pragma unroll
            for (int mm = 1; mm < k; ++mm) v = ff_subf(v, ff_mulf(ff_mulf(lK[mm], Lw[k][mm]), Dd[mm]));
            lK[k] = ff_divf(v, dk);
            logdet_G += ff_log(dk);
        }
        ff amin = ff_norm(A.GKKh, A.GKKl);
#pragma unroll
        for (int k = 1; k < L; ++k) amin = ff_subf(amin, ff_mulf(ff_mulf(lK[k], lK[k]), Dd[k]));
        const ff sK = ff_addf(amin, ff_make(ilam0, 0.f));
        ff zK = ff_norm(A.qKh, A.qKl);
        ff quad = ff_make(0.f, 0.f);
#pragma unroll
        for (int k = 1; k < L; ++k) {
            ff v = ff_norm(A.qTh[k], A.qTl[k]);
#pragma unroll
            for (int mm = 1; mm < k; ++mm) v = ff_subf(v, ff_mulf(Lw[k][mm], z[mm]));
            z[k] = v;
            quad = ff_addf(quad, ff_divf(ff_mulf(v, v), Dd[k]));
            zK = ff_subf(zK, ff_mulf(lK[k], v));
        }
        quad = ff_addf(quad, ff_divf(ff_mulf(zK, zK), sK));
        logdet_G += ff_log(sK);
        const ff chi2 = ff_subf(ff_norm(A.rh, A.rl), quad);
        const double slw = st.sum_log_ivar - 0.6931471805599453 * (double)A.lg2;
        lnl = -0.5 * (ff_to_d(chi2) + st.log_norm_rest + (double)log_lam0f + (double)logdet_G - slw);
        chi2f = chi2.hi;
        s_f = sK.hi;
        amin_f = amin.hi;
        Khat = zK.hi / sK.hi;
        quadf = quad.hi;
    }
    const float D = err_c0 * (1.0f + e) / (ome * ome);
    const float Wsum = st.sum_ivar;
    const float c2 = fmaxf(chi2f, 0.f);
    const float dchi = 2.f * fabsf(Khat) * D * sqrtf(Wsum * c2) + Khat * Khat * D * D * Wsum;
    const float ds = 2.f * D * sqrtf(Wsum * fmaxf(amin_f, 0.f)) + Wsum * D * D;
    const float room = s_f - ds;
    const float dlogs = (room > 1e-3f * s_f) ? ds / room : 1e30f;
    err = 0.5f * (dchi + dlogs) + 2e-6f + 2e-7f * (float)N +
          1e-12f * (fabsf(chi2f) + fabsf(quadf)) + (JIT ? 2e-7f * c2 : 0.f);
    if (!(err < 1e30f)) err = 1e30f;     // NaN inputs or overflow: no bound
                                         // (+infinity marks samples out of reach)
}

template <int L, bool JIT>
__device__ __forceinline__ Acc32<L, JIT, float> acc_lane(const Acc32<L, JIT, float2> &P, int lane) {
    Acc32<L, JIT, float> A;
    auto g = [lane](float2 v) { return lane ? v.y : v.x; };
    A.A00h = g(P.A00h); A.A00l = g(P.A00l); A.bh = g(P.bh); A.bl = g(P.bl);
    A.GKKh = g(P.GKKh); A.GKKl = g(P.GKKl); A.qKh = g(P.qKh); A.qKl = g(P.qKl);
    A.rh = g(P.rh); A.rl = g(P.rl); A.lg2 = g(P.lg2);
#pragma unroll
    for (int i = 0; i < MAXL; ++i) {
        A.Ah[i] = g(P.Ah[i]); A.Al[i] = g(P.Al[i]); A.GKh[i] = g(P.GKh[i]); A.GKl[i] = g(P.GKl[i]);
        A.qTh[i] = g(P.qTh[i]); A.qTl[i] = g(P.qTl[i]);
#pragma unroll
        for (int k = 0; k < MAXL; ++k) { A.GTh[i][k] = g(P.GTh[i][k]); A.GTl[i][k] = g(P.GTl[i][k]); }
    }
    return A;
}

// Load (or prepare, PACKED) sample `row` of the cache.
template <bool JIT, bool PACKED>
__device__ __forceinline__ void load_sample(const LnlArgs &a, int64_t row, float4 &pa, float4 &pb,
                                            float &s2) {
    if (PACKED) {
        const int64_t q = row * a.stride;
        prepare_sample(__ldg(a.P + q), __ldg(a.e + q), __ldg(a.om + q), __ldg(a.M0 + q),
                       JIT ? __ldg(a.s + q) : 0.0, pa, pb, s2);
    } else {
        pa = __ldg(a.mx_a + row);
        pb = __ldg(a.mx_b + row);
        s2 = JIT ? __ldg(a.mx_s2 + row) : 0.0f;
    }
}

// PACKED over the reference's interleaved chunk (P, e, omega, M0, s adjacent,
// stride 5): each pass stages its rows in shared memory with coalesced 8-byte
// loads (consecutive threads, consecutive doubles), so that a chunk in host
// memory read through a view crosses the link as whole lines, once.  Five
// strided loads per sample would fetch each line several times.
constexpr int PACK_ROWS = 256;          // rows per pass of the paired kernels

__device__ __forceinline__ bool packed_interleaved(const LnlArgs &a) {
    return a.stride == 5 && a.e == a.P + 1 && a.om == a.P + 2 && a.M0 == a.P + 3 &&
           a.s == a.P + 4;
}

// Rows [row, row + n) into smr; the caller synchronises before and after.
__device__ __forceinline__ void stage_rows(double *smr, const LnlArgs &a, int64_t row, int n) {
    const double *src = a.P + row * 5;
    for (int q = threadIdx.x; q < n * 5; q += blockDim.x) smr[q] = __ldg(src + q);
}

template <bool JIT>
__device__ __forceinline__ void prepare_row(const double *r, float4 &pa, float4 &pb, float &s2) {
    prepare_sample(r[0], r[1], r[2], r[3], JIT ? r[4] : 0.0, pa, pb, s2);
}

// The two samples of one pass of a paired kernel (thread t: samples base + t
// and base + blockDim + t of the work item): from staged rows over an
// interleaved chunk, else loaded directly.  Every thread of the CTA calls it.
template <bool JIT, bool PACKED>
__device__ __forceinline__ void load_pair(const LnlArgs &a, const WorkItem &w, int base,
                                          double *smr, bool inter, bool act0, bool act1,
                                          float4 &pa0, float4 &pb0, float &s20, float4 &pa1,
                                          float4 &pb1, float &s21) {
    const int j0 = base + threadIdx.x, j1 = j0 + blockDim.x;
    if (PACKED && inter) {
        __syncthreads();
        stage_rows(smr, a, w.row0 + base, min(2 * (int)blockDim.x, w.count - base));
        __syncthreads();
        prepare_row<JIT>(smr + 5 * (act0 ? (int)threadIdx.x : 0), pa0, pb0, s20);
        prepare_row<JIT>(smr + 5 * (act1 ? (int)(threadIdx.x + blockDim.x) : 0), pa1, pb1, s21);
    } else {
        load_sample<JIT, PACKED>(a, w.row0 + (act0 ? j0 : 0), pa0, pb0, s20);
        load_sample<JIT, PACKED>(a, w.row0 + (act1 ? j1 : 0), pa1, pb1, s21);
    }
}

__device__ __forceinline__ void store_sample(const LnlArgs &a, int64_t out, bool active, double lnl,
                                             float err, unsigned long long *mk,
                                             unsigned long long *bk) {
    if (active) {
        a.lnl[out] = lnl;
        if (a.err) a.err[out] = err;
    }
    if (mk) warp_max_update(mk, active ? double_to_key(lnl) : 0ull);
    if (bk) {
        warp_max_update(bk, active ? double_to_key(lnl + (double)err) : 0ull);
        warp_max_update(bk + 1, active ? double_to_key(lnl - (double)err) : 0ull);
    }
}

// One work item, one sample per thread: the star's epochs staged as REC32
// float records in smf (TILE epochs at a time).  *staged names the star whose
// records smf holds (a single-tile star stays staged across items).
template <int L, bool JIT, int VAR, bool PACKED>
__device__ __forceinline__ void mixed_item_scalar(const LnlArgs &a, const WorkItem &w,
                                                  float *smf, double *smr, int *staged) {
    const StarRec &st = a.stars[w.star];
    const int N = st.n_epochs;
    const bool single = N <= TILE;
    if (single && *staged != w.star) {
        stage_epochs<float, REC32>(smf, a.ep32 + (size_t)st.epoch_off * REC32, N);
        *staged = w.star;
        __syncthreads();
    }
    unsigned long long *mk = a.max_key ? a.max_key + w.max_slot : nullptr;
    unsigned long long *bk = a.bound_key ? a.bound_key + 2 * w.max_slot : nullptr;
    const bool mu0z = st.mu0_zero != 0;
    const float mu0f = st.mu0_f;
    const bool inter = PACKED && packed_interleaved(a);
    for (int base = 0; base < w.count; base += blockDim.x) {
        const int j = base + threadIdx.x;
        const bool active = j < w.count;
        float4 pa, pb;
        float s2;
        if (inter) {
            __syncthreads();
            stage_rows(smr, a, w.row0 + base, min((int)blockDim.x, w.count - base));
            __syncthreads();
            prepare_row<JIT>(smr + 5 * (active ? threadIdx.x : 0), pa, pb, s2);
        } else {
            load_sample<JIT, PACKED>(a, w.row0 + (active ? j : 0), pa, pb, s2);
        }
        const MixC<float> c = mix_consts(pa, pb, s2);
        Acc32<L, JIT, float> A;
        A.zero();
        for (int t0 = 0; t0 < N; t0 += TILE) {
            const int nt = min(TILE, N - t0);
            if (!single) {
                __syncthreads();
                stage_epochs<float, REC32>(smf, a.ep32 + ((size_t)st.epoch_off + t0) * REC32, nt);
                *staged = -1;
                __syncthreads();
            }
            if (active) {
#pragma unroll 2
                for (int i = 0; i < nt; ++i)
                    mixed_epoch<L, JIT, VAR == 1>(smf + i * REC32, c, mu0z, mu0f, -mu0f, A);
            }
        }
        double lnl = 0.0;
        float err = 0.0f;
        if (active) mixed_tail<L, JIT, VAR>(st, A, c.e, c.ome, pb.w, N, a.err_c0, lnl, err);
        store_sample(a, w.out_off + j, active, lnl, err, mk, bk);
    }
}

// One sample per thread (any L).
template <int L, bool JIT, int VAR, bool PACKED>
__global__ void __launch_bounds__(128)
lnl_mixed_kernel(LnlArgs a) {
    __shared__ __align__(16) float sm[TILE * REC32];
    __shared__ double smr[PACKED ? 128 * 5 : 1];
    __shared__ int s_item;
    int staged = -1;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.queue, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= item_count(a)) break;
        mixed_item_scalar<L, JIT, VAR, PACKED>(a, get_item(a, it), sm, smr, &staged);
    }
}

// Resident CTAs per SM the paired kernel is compiled for (its register cap).
#ifndef JOKER_PAIR_MINB
#define JOKER_PAIR_MINB 7
#endif

// Two samples per thread with paired FP32 arithmetic (L <= 3).  Thread t of a
// CTA evaluates samples base + t and base + blockDim + t of its work item.
template <int L, bool JIT, int VAR, bool PACKED>
__global__ void __launch_bounds__(128, JOKER_PAIR_MINB)
lnl_mixed2_kernel(LnlArgs a) {
    __shared__ __align__(16) float sm[TILE * REC32];
    __shared__ double smr[PACKED ? PACK_ROWS * 5 : 1];
    __shared__ int s_item;
    int staged_star = -1;
    const bool inter = PACKED && packed_interleaved(a);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.queue, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= item_count(a)) break;
        const WorkItem w = get_item(a, it);
        const StarRec &st = a.stars[w.star];
        const int N = st.n_epochs;
        const bool single = N <= TILE;
        if (single && w.star != staged_star) {
            stage_epochs<float, REC32>(sm, a.ep32 + (size_t)st.epoch_off * REC32, N);
            staged_star = w.star;
            __syncthreads();
        }
        unsigned long long *mk = a.max_key ? a.max_key + w.max_slot : nullptr;
        unsigned long long *bk = a.bound_key ? a.bound_key + 2 * w.max_slot : nullptr;
        const bool mu0z = st.mu0_zero != 0;
        const float2 mu0 = make_float2(st.mu0_f, st.mu0_f), nmu0 = make_float2(-st.mu0_f, -st.mu0_f);
        for (int base = 0; base < w.count; base += 2 * blockDim.x) {
            const int j0 = base + threadIdx.x, j1 = j0 + blockDim.x;
            const bool act0 = j0 < w.count, act1 = j1 < w.count;
            float4 pa0, pb0, pa1, pb1;
            float s20, s21;
            load_pair<JIT, PACKED>(a, w, base, smr, inter, act0, act1, pa0, pb0, s20, pa1, pb1,
                                   s21);
            const MixC<float> c0 = mix_consts(pa0, pb0, s20), c1 = mix_consts(pa1, pb1, s21);
            const MixC<float2> c = mix_pair(c0, c1);
            Acc32<L, JIT, float2> A;
            A.zero();
            for (int t0 = 0; t0 < N; t0 += TILE) {
                const int nt = min(TILE, N - t0);
                if (!single) {
                    __syncthreads();
                    stage_epochs<float, REC32>(sm, a.ep32 + ((size_t)st.epoch_off + t0) * REC32, nt);
                    staged_star = -1;
                    __syncthreads();
                }
                if (act0) {
#pragma unroll 2
                    for (int i = 0; i < nt; ++i)
                        mixed_epoch<L, JIT, VAR == 1>(sm + i * REC32, c, mu0z, mu0, nmu0, A);
                }
            }
            double lnl0 = 0.0, lnl1 = 0.0;
            float err0 = 0.0f, err1 = 0.0f;
            if (act0) mixed_tail<L, JIT, VAR>(st, acc_lane(A, 0), c0.e, c0.ome, pb0.w, N, a.err_c0, lnl0, err0);
            if (act1) mixed_tail<L, JIT, VAR>(st, acc_lane(A, 1), c1.e, c1.ome, pb1.w, N, a.err_c0, lnl1, err1);
            store_sample(a, w.out_off + j0, act0, lnl0, err0, mk, bk);
            store_sample(a, w.out_off + j1, act1, lnl1, err1, mk, bk);
        }
    }
}

// Persistent launch: as many CTAs as can be resident on the device (never more
// than there are work items); each CTA loops over the shared work counter.
// persistent_grid (joker_abi.cu) caches the grid per device, kernel and block.
cudaError_t persistent_grid(const void *kern, int block, int *grid);

template <typename K>
inline cudaError_t launch_persistent(K kern, const LnlArgs &a, int block, cudaStream_t st) {
    int grid = 0;
    cudaError_t e = persistent_grid(reinterpret_cast<const void *>(kern), block, &grid);
    if (e != cudaSuccess) return e;
    if (!a.n_items_dev && grid > a.n_items) grid = a.n_items;
    if (grid < 1) return cudaSuccess;
    kern<<<grid, block, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

}  // namespace joker

namespace joker {
// Paired form for L <= 3, and without jitter for any L (its epoch sums are
// L + 1 float pairs), unless JOKER_MIXED_PAIRED=0 (the one-sample-per-thread
// form, kept for comparison and for larger systems with jitter).
inline bool mixed_paired(int L, bool jit) {
    static int env = -1;
    if (env < 0) {
        const char *v = getenv("JOKER_MIXED_PAIRED");
        env = (v && v[0] == '0') ? 0 : 1;
    }
    return env == 1 && (L <= 3 || !jit);
}
}  // namespace joker
