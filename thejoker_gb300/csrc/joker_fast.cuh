// The FP32-sum ln L kernel (JOKER_MIXED_FAST): the first pass of the refined
// acceptance.  Same phase, FP32 Kepler and RV column as the mixed kernel,
// but every epoch sum is a plain FP32 accumulation, and each sample carries a
// rigorous bound err on |lnL - lnL_FP64| built from the sums' magnitudes.
//
// Re-centred sums.  With beta0 = C^-1 c the star's trend-only fit (any fixed
// shift would do) and r_c = y' - T^T beta0 its residual, for every sample
//   chi2 = r^T W r - q^T G^-1 q = C + beta0^T Lambda_T^-1 beta0 - q'^T G^-1 q',
//   C = r_c^T W r_c,  q' = M W r_c - Lambda^-1 (0, beta0),
// exactly (substitute r = r_c + T^T beta0).  The large terms of a systemic
// velocity never enter the FP32 sums: r_c is the scatter about the trend
// fit.  Since T W0 r_c = Lambda_T^-1 beta0 for the nominal weights
// W0 = diag(ivar),  q'_T = T (W - W0) r_c = -s^2 sum_i w_i ivar_i r_c,i T_i,
// one more product per term and no cancellation.  A K prior mean mu0 enters
// as r_c -> r_c - mu0 m, which the tail applies to the sums.  Without jitter
// the trend block and C + kappa = chi2_0 are folded on the host.
//
// Error bound.  A sequential FP32 sum of N terms, each with k roundings, is
// off by at most gamma sum |term|, gamma = (N + k) u / (1 - (N + k) u),
// u = 2^-24; the FP32 weight and the r_c, ivar r_c and T_j stored as floats
// are term-wise relative perturbations folded into k.  The magnitudes
// sum |term| come from the non-negative diagonal sums by Cauchy-Schwarz
// (sum |w m r_c| <= sqrt(F C), ...).  With theta = G^-1 q' (the best-fit
// linear parameters) and dq', dG the sums' errors,
//   d chi2 = dC - 2 theta.dq' + theta^T dG theta - (dq' - dG theta)^T
//            (G + dG)^-1 (dq' - dG theta),
// bounded term by term, the last by 2 tr(G^-1) |dq' - dG theta|^2 while
// |dG|_F tr(G^-1) < 1/4 (else err = 1e30: no bound, always refined); and
// |d log det G| <= |tr(G^-1 dG)| + 1.34 |G^-1 dG|_F^2.  The FP32 column's own
// error (FP32 Kepler and the phase's constant rounding: the empirical
// constant err_c0; the split phase's rounding, at most 2.5 2^-34 |dt| / P
// cycles, on top) enters as in the mixed kernel through its ivar-weighted
// norm, which by Minkowski's inequality takes the ivar-weighted RMS of |dt|
// in place of each epoch's |dt|.  The tail runs in float-float; the only FP64
// instruction per sample is the addition that rounds ln L's float pair to a
// double (both halves converted by integer operations).
#pragma once
#include "joker_mixed.cuh"

namespace joker {

constexpr float U32 = 5.9604645e-8f;    // 2^-24

template <int L, bool JIT, class T> struct AccF {
    T F, D, C, LG;                   // sum w m^2, sum w m r_c; jitter: sum w r_c^2, sum lg2(1+s^2 iv)
    T g[MAXL];                       // sum w m T_j (j >= 1)
    T Q[MAXL];                       // jitter: sum w ivar r_c T_j
    T G[MAXL][MAXL];                 // jitter: sum w T_j T_k (1 <= k <= j)
    __device__ __forceinline__ void zero() {
        const T z = vsplat<T>(0.0f);
        F = D = C = LG = z;
#pragma unroll
        for (int i = 0; i < MAXL; ++i) {
            g[i] = Q[i] = z;
#pragma unroll
            for (int k = 0; k < MAXL; ++k) G[i][k] = z;
        }
    }
};

// The unit-K RV column with a split phase: dt = dth + dtl with dth carrying
// 12 significant bits and 1/P = ih + il with ih carrying 12, so dth ih is
// exact in FP32 and so is its fractional part; |dth il| + |dtl / P| is below
// 2^-11 dt/P cycles, and the roundings of dtl, il, dtl 1/P, the FMA and the
// two additions of the phase leave at most 2.5 2^-34 dt/P cycles (1.2e-7
// cycles typically at dt/P = 2000: a 4000-day baseline at P = 2 d; the
// float-float phase of unit_rv_column gets 3e-8).  The bound adds that term,
// per sample from 1/P and the star's ivar-weighted RMS of |dt|, to the
// constant column error err_c0.  The reciprocal of the velocity's denominator is
// the hardware one (within 2^-23 relative, no Newton step).
template <bool SHIFT, class T>
__device__ __forceinline__ T unit_rv_column_split(T dth, T dtl, const MixC<T> &c) {
    const T p = vmul(dth, c.ih);                                          // exact
    const T fr = vsub(p, vrint<SHIFT>(p));                                // exact
    const T sm = vfma(dth, c.il, vmul(dtl, c.iph));
    const T f0 = vadd(vsub(fr, c.mch), vsub(sm, c.mcl));
    const T f = vsub(f0, vrint<SHIFT>(f0));                               // [-0.5, 0.5]
    const T M = vfma(f, vsplat<T>(TWO_PI_HI_F), vmul(f, vsplat<T>(TWO_PI_LO_F)));
    T sE, cE;
    vkepler<false>(M, c.e, c.ne, c.ome, c.ome3, c.a1, sE, cE);
    const T den = vfma(c.ne, cE, vsplat<T>(1.0f));
    const T rd = vmap([](float v) { return fast_rcp(v); }, den);
    return vfma(vfma(c.Ac, cE, vfma(c.Bc, sE, c.nDc)), rd, c.Dc);
}

// One epoch of the FP32-sum path.  Record words: 0,1 dt pair; 2 ivar;
// no jitter: 6 + 2 (j - 1) ivar T_j; jitter: 8 + 2 (j - 1) T_j; 16, 17 dt
// split as dth (12 significant bits) + dtl; 18 r_c; 19 ivar r_c.
template <int L, bool JIT, bool ACCURATE, class T>
__device__ __forceinline__ void fast_epoch(const float *recf, const MixC<T> &c,
                                           AccF<L, JIT, T> &A) {
    const T m = unit_rv_column_split<JIT>(vsplat<T>(recf[16]), vsplat<T>(recf[17]), c);
    const T iv = vsplat<T>(recf[2]);
    if constexpr (!JIT) {
        const T ivm = vmul(iv, m);
        A.F = vfma(ivm, m, A.F);
        A.D = vfma(vsplat<T>(recf[19]), m, A.D);
        if (L > 1) A.g[1] = vadd(A.g[1], ivm);
#pragma unroll
        for (int j = 2; j < L; ++j) A.g[j] = vfma(vsplat<T>(recf[6 + 2 * (j - 1)]), m, A.g[j]);
    } else {
        // w = ivar / (1 + s^2 ivar): one rounding for 1 + s^2 ivar, the
        // hardware reciprocal (within 2^-23 relative) and the product
        const T onep = vfma(c.s2, iv, vsplat<T>(1.0f));
        const T w = vmul(iv, vmap([](float v) { return fast_rcp(v); }, onep));
        A.LG = vadd(A.LG, vmap([](float v) { return lg2_approx(v); }, onep));
        const T rc = vsplat<T>(recf[18]);
        const T wm = vmul(w, m);
        A.F = vfma(wm, m, A.F);
        A.D = vfma(wm, rc, A.D);
        const T wr = vmul(w, rc);
        A.C = vfma(wr, rc, A.C);
        const T wq = vmul(w, vsplat<T>(recf[19]));
        if (L > 1) {
            A.g[1] = vadd(A.g[1], wm);
            A.G[1][1] = vadd(A.G[1][1], w);
            A.Q[1] = vadd(A.Q[1], wq);
        }
#pragma unroll
        for (int j = 2; j < L; ++j) {
            const T Tj = vsplat<T>(recf[8 + 2 * (j - 1)]);
            A.g[j] = vfma(wm, Tj, A.g[j]);
            A.Q[j] = vfma(wq, Tj, A.Q[j]);
            const T wt = vmul(w, Tj);
            A.G[j][1] = vadd(A.G[j][1], wt);
#pragma unroll
            for (int k = 2; k <= j; ++k)
                A.G[j][k] = vfma(wt, vsplat<T>(recf[8 + 2 * (k - 1)]), A.G[j][k]);
        }
    }
}

__device__ __forceinline__ ff ffv(float x) { return ff_make(x, 0.0f); }

// The per-sample tail: ln L as a float pair (hi, lo) and its bound err.
//
// With H the trend block of G (Lambda_T^-1 + T W T^T: folded on the host
// without jitter, from the sums with it), v = H^-1 g, s = 1/Lambda0 + F -
// g^T v, q'_K = D - mu0 F, q'_T = -s^2 Q - mu0 g (no Q without jitter),
// z = H^-1 q'_T and t = q'_K - g^T z:
//   chi2 = C_eff - q'_T^T z - t^2 / s,  theta_K = t / s,  theta_T = z - v theta_K,
//   C_eff = C + kappa - 2 mu0 D + mu0^2 F   (chi2_0 in place of C + kappa
//                                            without jitter),
//   log det G = log det H + log s.
template <int L, bool JIT>
__device__ __forceinline__ void fast_tail(const StarRec &st, const AccF<L, JIT, float> &A,
                                          float e, float ome, float lgP, float s2, int N,
                                          float err_c0, ff &lnl, float &err) {
    constexpr int T = L - 1;
    static_assert(!JIT || L <= 3, "the FP32-sum path takes at most three linear parameters "
                                  "with the jitter applied");
    // (the float copies of the prior's logs: no FP64 conversion per sample)
    const float log_lam0f =
        st.k_scaled ? fminf(st.log_maxK2_f, st.log_kscale_f + lgP) : st.log_lam0_f;
    const float ilam0 = expf(-log_lam0f);
    const float mu = st.mu0_f, amu = fabsf(mu);
    // gamma: sequential FP32 sums of N terms; per term the FP32 weight (4
    // roundings with jitter), the products, and r_c, ivar r_c, T_j as floats
    const float gam = __fmul_ru((float)(N + (JIT ? 7 : 4)), U32) * 1.0001f;
    const float F = A.F, D = A.D;
    // ---- trend block inverse Hi and log det H
    ff Hi[MAXL][MAXL];
    ff ldH = ffv(0.0f);
    if constexpr (!JIT) {
#pragma unroll
        for (int j = 0; j < T; ++j)
#pragma unroll
            for (int k = 0; k < T; ++k)
                Hi[j][k] = ff_make(st.Cinv_hi[(j + 1) * MAXL + k + 1],
                                   st.Cinv_lo[(j + 1) * MAXL + k + 1]);
    } else if constexpr (T == 1) {
        const ff H11 = ff_addf(ffv(A.G[1][1]), ff_make(st.ilam_hi[1], st.ilam_lo[1]));
        Hi[0][0] = ff_divf(ffv(1.0f), H11);
        ldH = ffv(ff_log(H11));
    } else if constexpr (T == 2) {
        const ff H11 = ff_addf(ffv(A.G[1][1]), ff_make(st.ilam_hi[1], st.ilam_lo[1]));
        const ff H21 = ffv(A.G[2][1]);
        const ff H22 = ff_addf(ffv(A.G[2][2]), ff_make(st.ilam_hi[2], st.ilam_lo[2]));
        const ff det = ff_subf(ff_mulf(H11, H22), ff_mulf(H21, H21));
        const ff idet = ff_divf(ffv(1.0f), det);
        Hi[0][0] = ff_mulf(H22, idet);
        Hi[1][1] = ff_mulf(H11, idet);
        Hi[0][1] = Hi[1][0] = ff_neg(ff_mulf(H21, idet));
        ldH = ffv(ff_log(det));
    }
    // ---- v = Hi g, q'_T, z = Hi q'_T
    float qT[MAXL];
#pragma unroll
    for (int j = 0; j < T; ++j) qT[j] = (JIT ? -s2 * A.Q[j + 1] : 0.0f) - mu * A.g[j + 1];
    ff v[MAXL], z[MAXL];
    ff gv = ffv(0.0f), gz = ffv(0.0f), qz = ffv(0.0f);
#pragma unroll
    for (int j = 0; j < T; ++j) {
        v[j] = ffv(0.0f);
        z[j] = ffv(0.0f);
#pragma unroll
        for (int k = 0; k < T; ++k) {
            v[j] = ff_addf(v[j], ff_mul1(Hi[j][k], A.g[k + 1]));
            z[j] = ff_addf(z[j], ff_mul1(Hi[j][k], qT[k]));
        }
    }
#pragma unroll
    for (int j = 0; j < T; ++j) {
        gv = ff_addf(gv, ff_mul1(v[j], A.g[j + 1]));
        gz = ff_addf(gz, ff_mul1(z[j], A.g[j + 1]));
        qz = ff_addf(qz, ff_mul1(z[j], qT[j]));
    }
    const ff amin = ff_subf(ffv(F), gv);                 // s - 1/Lambda0
    const ff s = ff_addf(amin, ffv(ilam0));
    const ff tK = ff_subf(ff_subf(ffv(D), ff_mul1(ffv(F), mu)), gz);
    const ff K = ff_divf(tK, s);                         // theta_K
    ff Ceff = JIT ? ff_addf(ffv(A.C), ff_make(st.kappa_hi, st.kappa_lo))
                  : ff_make(st.chi2_0_hi, st.chi2_0_lo);
    if (mu != 0.0f) Ceff = ff_addf(Ceff, ff_mul1(ff_subf(ff_mul1(ffv(F), mu), ffv(2.0f * D)), mu));
    const ff chi2 = ff_subf(ff_subf(Ceff, qz), ff_mulf(K, tK));
    const float chi2f = chi2.hi, sf = s.hi, Kh = fabsf(K.hi);
    float th[MAXL];
#pragma unroll
    for (int j = 0; j < T; ++j) th[j] = fabsf(z[j].hi - v[j].hi * K.hi);
    // ---- rounding of the sums: magnitudes by Cauchy-Schwarz from the
    // non-negative sums (F, C, the diagonal trend sums)
    const float Cmag = JIT ? A.C : st.Cn;
    const float dF = gam * F;
    const float dD = gam * sqrtf(F * Cmag);
    float Gjj[MAXL], dg[MAXL], aT[MAXL];
#pragma unroll
    for (int j = 0; j < T; ++j) {
        Gjj[j] = JIT ? A.G[j + 1][j + 1] : st.Wjj[j + 1];
        dg[j] = gam * sqrtf(F * Gjj[j]);
        aT[j] = amu * dg[j];
        if (JIT)
            aT[j] += s2 * (gam * sqrtf(Gjj[j]) * sqrtf(A.C) * st.ivar_max +
                           U32 * sqrtf(st.Cn * st.Wjj[j + 1])) + U32 * fabsf(qT[j]);
    }
    const float aK = dD + amu * dF;
    const float dC = (JIT ? gam * A.C : 0.0f) + 2.0f * amu * dD + mu * mu * dF;
    // The second-order terms are taken in the frame scaled by D = diag(d_i),
    // d_i^2 ~ G_ii (any positive diagonal is valid; this one makes the
    // terms independent of the columns' units, e.g. a (t - t_ref)^2 trend
    // column in days^2): with G~ = D^-1 G D^-1, dG~ = D^-1 dG D^-1 and
    // r~ = D^-1 (dq' - dG theta), (dq' - dG theta)^T (G + dG)^-1 (...) =
    // r~^T (G~ + dG~)^-1 r~ <= 2 tr(G~^-1) |r~|^2 while |dG~|_F tr(G~^-1) <= 1/2,
    // and G^-1 dG is similar to G~^-1 dG~, whose Frobenius norm is at most
    // |dG~|_F tr(G~^-1).  Each entry of dG~ is at most gam.
    // (hardware reciprocals of the scales: their 2^-23 relative error is
    // inside the bound's 1 % evaluation allowance)
    const float dK2 = F + ilam0, idK2 = fast_rcp(dK2);
    float dT2[MAXL], idT2[MAXL];
#pragma unroll
    for (int j = 0; j < T; ++j) {
        dT2[j] = fmaxf(Gjj[j] + st.ilam_hi[j + 1], 1e-30f);   // H_jj
        idT2[j] = fast_rcp(dT2[j]);
    }
    // first order: dC + 2 |theta|.|dq'| + |theta|^T |dG| |theta|
    float d1 = dC + 2.0f * Kh * aK + Kh * Kh * dF;
    float eK = aK + Kh * dF;
    float dGs2 = (dF * idK2) * (dF * idK2);           // |dG~|_F^2
    float eT[MAXL];
#pragma unroll
    for (int j = 0; j < T; ++j) {
        d1 += 2.0f * th[j] * (aT[j] + Kh * dg[j]);
        eK += th[j] * dg[j];
        eT[j] = aT[j] + Kh * dg[j];
        dGs2 += 2.0f * (dg[j] * dg[j]) * (idK2 * idT2[j]);
    }
    if constexpr (JIT) {
#pragma unroll
        for (int j = 0; j < T; ++j)
#pragma unroll
            for (int k = 0; k < T; ++k) {
                const float dG = gam * sqrtf(Gjj[j] * Gjj[k]);
                d1 += th[j] * th[k] * dG;
                eT[j] += dG * th[k];
                dGs2 += (dG * dG) * (idT2[j] * idT2[k]);
            }
    }
    // second order: 2 tr(G~^-1) |r~|^2, valid while |dG~|_F tr(G~^-1) < 1/4;
    // (G^-1)_KK = 1/s and (G^-1)_jj = (H^-1)_jj + v_j^2 / s
    const float iS = fast_rcp(sf);
    float trGi = iS * dK2;
#pragma unroll
    for (int j = 0; j < T; ++j) trGi += (Hi[j][j].hi + v[j].hi * v[j].hi * iS) * dT2[j];
    float ee = eK * eK * idK2;
#pragma unroll
    for (int j = 0; j < T; ++j) ee += eT[j] * eT[j] * idT2[j];
    const float xf = sqrtf(dGs2) * trGi;
    bool ok = xf < 0.25f;
    d1 += 2.0f * trGi * ee;
    // log det G: |tr(G^-1 dG)| + 1.34 |G^-1 dG|_F^2
    float dl = iS * dF;
#pragma unroll
    for (int j = 0; j < T; ++j) dl += 2.0f * fabsf(v[j].hi) * iS * dg[j];
    if constexpr (JIT) {
#pragma unroll
        for (int j = 0; j < T; ++j)
#pragma unroll
            for (int k = 0; k < T; ++k)
                dl += fabsf(Hi[j][k].hi + v[j].hi * v[k].hi * iS) * gam * sqrtf(Gjj[j] * Gjj[k]);
    }
    float dlog = dl + 1.34f * xf * xf;
    // ---- the FP32 column's own error (err_c0: the empirical constant plus
    // the phase term of this sample, as in the mixed kernel): chi2 is a minimum over the linear parameters, so it moves by
    // -2 K sum w res dm; s moves directly
    const float Dcol = err_c0 * (1.0f + e) / (ome * ome);
    const float Wsum = st.sum_ivar;
    const float c2 = fmaxf(chi2f, 0.0f);
    const float dsc = 2.0f * Dcol * sqrtf(Wsum * fmaxf(amin.hi, 0.0f)) + Wsum * Dcol * Dcol;
    ok = ok && dsc < 0.5f * sf;
    float dchi = d1 + 2.0f * Kh * Dcol * sqrtf(Wsum * c2) + Kh * Kh * Dcol * Dcol * Wsum;
    dlog += dsc / (sf - dsc);
    if constexpr (JIT) {
        // r_c stored as floats is a data perturbation; the FP32 log2 sum
        dchi += 2.0f * U32 * sqrtf(c2 * st.Cn) + U32 * U32 * st.Cn;
        dlog += gam * A.LG * 0.6931472f;
    }
    // ---- ln L
    ff t;
    if constexpr (!JIT) {
        // -(chi2 + logdet_const + log Lambda0 + log s) / 2
        t = ff_addf(chi2, ff_make(st.ldc_hi, st.ldc_lo));
    } else {
        // -(chi2 + log_norm_rest - sum log ivar + log Lambda0 + log det H + log s
        //   + ln 2 sum lg2(1 + s^2 ivar)) / 2
        t = ff_addf(chi2, ff_make(st.lnr_hi, st.lnr_lo));
        t = ff_addf(t, ldH);
        t = ff_addf(t, ff_mul1(ffv(A.LG), 0.6931472f));
    }
    t = ff_addf(t, ffv(log_lam0f));
    t = ff_addf(t, ffv(ff_log(s)));
    lnl = ff_make(-0.5f * t.hi, -0.5f * t.lo);
    const float tailmag = fabsf(Ceff.hi) + fabsf(qz.hi) + Kh * fabsf(tK.hi);
    // plus: log Lambda0 and the logs of the tail in FP32 (2e-6), the FP32 log2
    // of each epoch's jitter term (2e-7 N), the float-float tail (its terms'
    // magnitude times 2^-40), and 1 % for the FP32 evaluation of the bound
    err = 1.01f * (0.5f * (dchi + dlog) + 2e-6f + 2e-7f * (float)N + 1e-12f * tailmag);
    // no bound: 1e30 (+infinity is reserved for samples out of reach)
    if (!ok || !(err < 1e30f) || !(lnl.hi == lnl.hi)) err = 1e30f;
}

template <int L, bool JIT>
__device__ __forceinline__ AccF<L, JIT, float> accf_lane(const AccF<L, JIT, float2> &P, int lane) {
    AccF<L, JIT, float> A;
    auto g = [lane](float2 v) { return lane ? v.y : v.x; };
    A.F = g(P.F); A.D = g(P.D); A.C = g(P.C); A.LG = g(P.LG);
#pragma unroll
    for (int i = 0; i < MAXL; ++i) {
        A.g[i] = g(P.g[i]);
        A.Q[i] = g(P.Q[i]);
#pragma unroll
        for (int k = 0; k < MAXL; ++k) A.G[i][k] = g(P.G[i][k]);
    }
    return A;
}

// Order-preserving key of the double equal to a float, from the float's bits
// (integer operations only).
__device__ __forceinline__ unsigned long long float_to_dkey(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned ex = (b >> 23) & 0xff;
    const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
    unsigned long long d;
    if (ex == 0xff) {
        d = sign | 0x7ff0000000000000ull | ((unsigned long long)(b & 0x7fffffu) << 29);
    } else if (ex == 0) {
        d = sign;                       // zero or subnormal: +-0
    } else {
        d = sign | ((unsigned long long)(ex + 896) << 52) |
            ((unsigned long long)(b & 0x7fffffu) << 29);
    }
    return key_of_bits((long long)d);
}

// The double equal to a float, from the float's bits (integer operations:
// the conversion instruction would occupy the FP64 pipe, 1/64 of the FP32
// rate on this GPU).  Zero, subnormal, infinite and NaN inputs convert as
// usual.
__device__ __forceinline__ double f2d_exact(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned ex = (b >> 23) & 0xffu;
    if (ex - 1u < 254u)
        return __longlong_as_double((long long)(((unsigned long long)(b & 0x80000000u) << 32) |
                                                ((unsigned long long)(ex + 896u) << 52) |
                                                ((unsigned long long)(b & 0x7fffffu) << 29)));
    if ((b & 0x7fffffffu) == 0u)
        return __longlong_as_double((long long)((unsigned long long)b << 32));   // +-0
    return (double)x;
}

// A key's double rounded down to a float: the bit pattern directly when the
// double is a normal float (bound keys are written from floats), else the
// FP64 conversion.
__device__ __forceinline__ float key_to_float_rd(unsigned long long k) {
    const unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
    const unsigned ex = (unsigned)(b >> 52) & 0x7ffu;
    if ((b & 0x1FFFFFFFull) == 0ull && ex >= 897u && ex <= 1150u)
        return __uint_as_float(((unsigned)(b >> 32) & 0x80000000u) | ((ex - 896u) << 23) |
                               ((unsigned)(b >> 29) & 0x7fffffu));
    return __double2float_rd(__longlong_as_double((long long)b));
}

__device__ __forceinline__ unsigned long long warp_max_key(unsigned long long k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, k, o);
        k = other > k ? other : k;
    }
    return k;
}

__device__ __forceinline__ void key_max_update(unsigned long long *key, unsigned long long k) {
    if ((threadIdx.x & 31) == 0 && k != 0ull) {
        if (k > *((volatile unsigned long long *)key)) atomicMax(key, k);
    }
}

// Both samples of a pass: ln L (and its bound) written out, the running
// maxima raised (one warp reduction each, over both samples).  Returns the
// warp's largest lower bound lnL - err as a key (0: none).
__device__ __forceinline__ unsigned long long fast_store2(const LnlArgs &a, int64_t out0,
                                                          bool act0, ff l0, float e0,
                                                          int64_t out1, bool act1, ff l1,
                                                          float e1, unsigned long long *mk,
                                                          unsigned long long *bk) {
    double d0 = 0.0, d1 = 0.0;
    if (act0) {
        d0 = f2d_exact(l0.hi) + f2d_exact(l0.lo);
        a.lnl[out0] = d0;
        if (a.err) a.err[out0] = e0;
    }
    if (act1) {
        d1 = f2d_exact(l1.hi) + f2d_exact(l1.lo);
        a.lnl[out1] = d1;
        if (a.err) a.err[out1] = e1;
    }
    auto kmax = [](unsigned long long x, unsigned long long y) { return x > y ? x : y; };
    if (mk)
        key_max_update(mk, warp_max_key(kmax(act0 ? double_to_key(d0) : 0ull,
                                             act1 ? double_to_key(d1) : 0ull)));
    unsigned long long kd = 0ull;
    if (bk) {
        // lnL + err rounded up and lnL - err rounded down, as floats
        const float up0 = __fadd_ru(l0.hi, __fadd_ru(l0.lo, e0));
        const float dn0 = __fadd_rd(l0.hi, __fsub_rd(l0.lo, e0));
        const float up1 = __fadd_ru(l1.hi, __fadd_ru(l1.lo, e1));
        const float dn1 = __fadd_rd(l1.hi, __fsub_rd(l1.lo, e1));
        key_max_update(bk, warp_max_key(kmax(act0 ? float_to_dkey(up0) : 0ull,
                                             act1 ? float_to_dkey(up1) : 0ull)));
        kd = warp_max_key(kmax(act0 ? float_to_dkey(dn0) : 0ull, act1 ? float_to_dkey(dn1) : 0ull));
        key_max_update(bk + 1, kd);
    }
    return kd;
}

// ---- the fused first acceptance pass
// Thread 0 of the block, at the start of a work item: the generator state
// before the item's first uniform and every 256 samples after it (the block's
// passes), the increment, and the 128-step constant S_128 inc.  Shared
// layout: s[2p], s[2p + 1] pass p (lo, hi); then inc, then S_128 inc.
constexpr int FUSED_PASSES = FUSED_MAX_CHUNK / 256;

__device__ __forceinline__ void fused_item_states(const LnlArgs &a, const WorkItem &w,
                                                  unsigned long long *s) {
    const unsigned long long *g = a.fa_pcg + 4 * (int64_t)w.max_slot;
    const u128 inc = ((u128)g[2] << 64) | (u128)g[3];
    u128 x = pcg_jump(((u128)g[0] << 64) | (u128)g[1], inc,
                      (uint64_t)(a.fa_first + (w.row0 - a.row0)));
    const u128 A256 = u128_of(g_pcg.dbl_a[8]), C256 = u128_of(g_pcg.dbl_s[8]) * inc;
    const int np = (w.count + 255) >> 8;
    for (int p = 0; p < np; ++p) {
        s[2 * p] = (unsigned long long)x;
        s[2 * p + 1] = (unsigned long long)(x >> 64);
        x = A256 * x + C256;
    }
    const u128 C128 = u128_of(g_pcg.dbl_s[7]) * inc;
    s[2 * FUSED_PASSES] = (unsigned long long)inc;
    s[2 * FUSED_PASSES + 1] = (unsigned long long)(inc >> 64);
    s[2 * FUSED_PASSES + 2] = (unsigned long long)C128;
    s[2 * FUSED_PASSES + 3] = (unsigned long long)(C128 >> 64);
}

// A sample can be accepted only if exp(lnL_64 - max) > u.  With lb the
// running lower bound of the maximum (lb <= max) and lnL_64 <= lnl + err, a
// sample with lnl + err - lb < log u is rejected whatever the maximum; every
// other sample is a candidate, including each one that can be the maximum
// (lnl + err >= max >= lb).  The float test keeps a margin for the FP32 log
// of u and for the float forms of lnl and lb, as the acceptance scan does.
//
// Most samples need no uniform: x = lnl + err - lb (with the margin) >= 0
// makes a candidate for any u < 1, and x < -746 rejects for every u,
// u = 0 included (exp of anything below -745.2 is 0 in FP64).  Returns 0
// (rejected), 1 (candidate) or 2 (test against u).
__device__ __forceinline__ int fused_pretest(bool act, ff l, float err, bool lb_ok, float lbf,
                                             float &x) {
    x = 0.0f;
    if (!act) return 0;
    if (!(err < 1e29f) || !(l.hi == l.hi) || !lb_ok) return 1;
    const float tol = 1e-4f + 5e-7f * (fabsf(l.hi) + fabsf(lbf) + err);
    x = (l.hi - lbf) + err + tol;
    if (x >= 0.0f) return 1;
    if (x < -746.0f) return 0;
    return 2;
}

// The test against u = m 2^-53 of a sample that fused_pretest left open.
__device__ __forceinline__ int fused_utest(int c, float x, uint64_t m) {
    if (c != 2) return c;
    if (m == 0ull) return 1;                          // u = 0: decided in FP64 later
    return x < __logf(u53_to_float(m)) ? 0 : 1;
}

// The warp's two candidate words of a pass (lanes on j0 = base + t and on
// j1 = j0 + 128), written by lane 0 for the words inside the item.
__device__ __forceinline__ void fused_write_words(const LnlArgs &a, const WorkItem &w, int base,
                                                  unsigned b0, unsigned b1) {
    if ((threadIdx.x & 31) == 0) {
        const int wo = base + (int)(threadIdx.x & ~31u);          // the warp's first j0
        const int64_t q = a.fa_first + (w.row0 - a.row0) + wo;    // its stream position
        uint32_t *cw = a.cand_words + (int64_t)w.max_slot * a.cand_ld + (q >> 5);
        if (wo < w.count) cw[0] = b0;
        if (wo + 128 < w.count) cw[4] = b1;
    }
}

template <bool FUSED>
__device__ __forceinline__ void fused_pass(const LnlArgs &a, const WorkItem &w, int base,
                                           const unsigned long long *s, unsigned long long kd,
                                           const unsigned long long *bk, bool act0, ff l0,
                                           float e0, bool act1, ff l1, float e1) {
    if constexpr (FUSED) {
        // the running lower bound: this warp's, or the slot's if larger
        const unsigned long long gk = *((volatile const unsigned long long *)(bk + 1));
        const unsigned long long lk = gk > kd ? gk : kd;
        const bool lb_ok = lk != 0ull && lk != 0xFFFFFFFFFFFFFFFFull;   // a bound, not NaN
        const float lbf = lb_ok ? key_to_float_rd(lk) : 0.0f;
        float x0, x1;
        int c0 = fused_pretest(act0, l0, e0, lb_ok, lbf, x0);
        int c1 = fused_pretest(act1, l1, e1, lb_ok, lbf, x1);
        if (__any_sync(0xffffffffu, c0 == 2 || c1 == 2)) {
            // the uniforms of j0 and j1 = j0 + 128 from the pass's state
            const int p = base >> 8;
            const u128 sb = ((u128)s[2 * p + 1] << 64) | (u128)s[2 * p];
            const u128 inc = ((u128)s[2 * FUSED_PASSES + 1] << 64) | (u128)s[2 * FUSED_PASSES];
            const u128 C128 =
                ((u128)s[2 * FUSED_PASSES + 3] << 64) | (u128)s[2 * FUSED_PASSES + 2];
            const u128 st0 = pcg_thread_step(sb, inc, threadIdx.x);
            const u128 st1 = u128_of(g_pcg.dbl_a[7]) * st0 + C128;
            c0 = fused_utest(c0, x0, pcg_output(st0) >> 11);
            c1 = fused_utest(c1, x1, pcg_output(st1) >> 11);
        }
        const unsigned b0 = __ballot_sync(0xffffffffu, c0 == 1);
        const unsigned b1 = __ballot_sync(0xffffffffu, c1 == 1);
        fused_write_words(a, w, base, b0, b1);
    }
}

// ---- early exit of the fused pass (L <= 3, stars of one epoch tile)
// ln L over all N epochs is at most the same expression over the first k
// epochs, with the unseen epochs' log weights taken at their largest,
// log ivar: chi2 over k epochs minimised over the linear parameters is at
// most chi2 over all of them (terms are only added), and log det G only grows
// as epochs are added (G_N - G_k is positive semi-definite).  With the
// re-centred sums the k-epoch chi2 is C_k + kappa - q'_k^T G_k^-1 q'_k (the
// substitution r = r_c + T^T beta0 holds on any subset of epochs), where
// q'_T = P_k - s^2 Q_k - mu0 g_k and P_k (per checkpoint, from the host)
// carries sum_{i<k} ivar r_c T - Lambda_T^-1 beta0; without jitter the
// trend block's inverse and log det come from the host as well.
//
// Returns -1/2 of the k-epoch expression and in dub a margin for its error:
// 1e-3 of its terms' magnitudes (over 100 times the rounding of FP32 sums of
// at most 103 terms, which covers the cross sums' Cauchy-Schwarz factors in
// practice; 100 (k + 3) 2^-24 for longer sums), plus the amplification of the sums' rounding through an
// ill-conditioned Schur complement s or trend block H (t^2 / s and
// q'^T H^-1 q' move by their relative errors), plus twice the FP32 column's
// own error term of the full bound (err_c0 (1 + e) / (1 - e)^2 per epoch,
// large for eccentric orbits), and 2 nats; valid = false when s or det H
// lies within four times its error of zero (a long-period sample nearly
// collinear with the constant column, say).
template <int L, bool JIT>
__device__ __forceinline__ float fast_upper(const StarRec &st, const AccF<L, JIT, float> &A,
                                            const float *ck, int nsum, float lgP, float s2,
                                            float e, float ome, float err_c0, float &dub,
                                            bool &valid) {
    constexpr int T = L - 1;
    constexpr int TT = T > 0 ? T : 1;
    static_assert(L <= 3 || (L == 4 && !JIT),
                  "the upper bound takes at most three linear parameters, four without jitter");
    // g1: three times the rounding bound of an FP32 sum of nsum terms (at
    // least that of 103 terms); fm: over 100 times that bound
    const float nu = (float)(nsum + 3) * U32;
    const float g1 = fmaxf(2e-5f, 3.0f * nu);
    const float fm = fmaxf(1e-3f, 100.0f * nu);
    const float log_lam0f =
        st.k_scaled ? fminf(st.log_maxK2_f, st.log_kscale_f + lgP) : st.log_lam0_f;
    const float ilam0 = __expf(-log_lam0f);
    const float mu = st.mu0_f;
    float Hi[TT][TT], ldH = 0.0f, rH = 0.0f;
#pragma unroll
    for (int j = 0; j < TT; ++j)
#pragma unroll
        for (int m = 0; m < TT; ++m) Hi[j][m] = 0.0f;
    valid = true;
    if constexpr (!JIT) {
        // host-computed: only the float rounding of the entries (three trend
        // columns: all epochs only, the third row of C^-1 in the P slots)
        if (T >= 1) Hi[0][0] = ck[3];
        if (T >= 2) { Hi[0][1] = Hi[1][0] = ck[4]; Hi[1][1] = ck[5]; }
        if (T == 3) {
            Hi[0][2] = Hi[2][0] = ck[0];
            Hi[1][2] = Hi[2][1] = ck[1];
            Hi[2][2] = ck[7];
        }
        ldH = ck[6];
        rH = 1e-6f;
    } else if constexpr (T == 1) {
        const float H11 = A.G[1][1] + st.ilam_hi[1];
        Hi[0][0] = 1.0f / H11;
        ldH = __logf(H11);
        rH = 2.0f * g1;
        valid = H11 > 0.0f;
    } else if constexpr (T == 2) {
        const float H11 = A.G[1][1] + st.ilam_hi[1], H21 = A.G[2][1];
        const float H22 = A.G[2][2] + st.ilam_hi[2];
        const float det = H11 * H22 - H21 * H21;
        const float ddet = 2.0f * g1 * (H11 * H22 + H21 * H21);
        const float idet = 1.0f / det;
        Hi[0][0] = H22 * idet; Hi[1][1] = H11 * idet; Hi[0][1] = Hi[1][0] = -H21 * idet;
        ldH = __logf(det);
        rH = ddet / (det - ddet) + g1;
        valid = det > 4.0f * ddet && H11 > 0.0f;
    }
    float g[TT], qT[TT];
#pragma unroll
    for (int j = 0; j < T; ++j) {
        g[j] = A.g[j + 1];
        qT[j] = (T == 3 ? 0.0f : ck[j]) - (JIT ? s2 * A.Q[j + 1] : 0.0f) - mu * g[j];
    }
    float gv = 0.0f, gz = 0.0f, qz = 0.0f;
#pragma unroll
    for (int j = 0; j < T; ++j) {
        float vj = 0.0f, zj = 0.0f;
#pragma unroll
        for (int m = 0; m < T; ++m) {
            vj += Hi[j][m] * g[m];
            zj += Hi[j][m] * qT[m];
        }
        gv += g[j] * vj;
        gz += g[j] * zj;
        qz += qT[j] * zj;
    }
    const float sK = A.F - gv + ilam0;
    const float ds = g1 * (A.F + ilam0 + fabsf(gv)) + rH * fabsf(gv);
    const float tK = A.D - mu * A.F - gz;
    float Ceff = JIT ? A.C + st.kappa_hi : ck[2];
    if (mu != 0.0f) Ceff += mu * (mu * A.F - 2.0f * A.D);
    const float q2 = tK * tK / sK;
    const float chi2 = Ceff - qz - q2;
    const float lnr = st.lnr_hi;
    const float lsK = __logf(sK);
    float t = chi2 + lnr + ldH + log_lam0f + lsK;
    if (JIT) t += 0.6931472f * A.LG;
    const float mag = fabsf(Ceff) + fabsf(qz) + q2 + fabsf(lnr) + fabsf(ldH) +
                      fabsf(log_lam0f) + fabsf(lsK) + (JIT ? 0.6931472f * A.LG : 0.0f);
    // the FP32 column's own error (err_c0, as in the full bound): chi2 moves
    // by at most 2 |theta_K| Dcol sqrt(W chi2) + theta_K^2 Dcol^2 W, s by dsc
    const float Dcol = err_c0 * (1.0f + e) / (ome * ome);
    const float Wsum = st.sum_ivar, Kh = fabsf(tK / sK), c2 = fmaxf(chi2, 0.0f);
    const float dsc = 2.0f * Dcol * sqrtf(Wsum * fmaxf(A.F - gv, 0.0f)) + Wsum * Dcol * Dcol;
    valid = valid && sK > 4.0f * ds && dsc < 0.5f * sK && (t == t) && mag < 1e30f;
    const float col = 2.0f * Kh * Dcol * sqrtf(Wsum * c2) + Kh * Kh * Dcol * Dcol * Wsum +
                      dsc / (sK - dsc);
    const float cond = q2 * ds / (sK - ds) + fabsf(qz) * rH + ds / (sK - ds) + rH * (float)T;
    dub = 0.5f * (fm * mag + 2.0f * cond + 2.0f * col) + 2.0f;
    return -0.5f * t;
}

// Whether every active sample of the warp is out of reach after the first
// nsum epochs (ck: that checkpoint's constants, or ck_full after all of them):
// its upper bound plus its margin lies more than 746 nats below the running
// lower bound of the maximum.  Such a sample is
// rejected for every uniform, 0 included, and cannot be the maximum.  ub0
// and ub1 receive the lanes' bounds.
template <int L, bool JIT>
__device__ __forceinline__ bool warp_out_of_reach(const StarRec &st,
                                                  const AccF<L, JIT, float2> &A,
                                                  const float *ck, int nsum, float e0,
                                                  float ome0, float e1, float ome1, float lgP0,
                                                  float lgP1, float s20, float s21, float ec0,
                                                  float ec1, bool act0, bool act1,
                                                  const unsigned long long *bk, float &ub0,
                                                  float &ub1) {
    const unsigned long long gk = *((volatile const unsigned long long *)(bk + 1));
    const bool lb_ok = gk != 0ull && gk != 0xFFFFFFFFFFFFFFFFull;
    bool h0 = !act0, h1 = !act1;
    ub0 = ub1 = 0.0f;
    if (__any_sync(0xffffffffu, lb_ok)) {
        const float lim = (lb_ok ? key_to_float_rd(gk) : 0.0f) - 746.0f;
        float dub;
        bool ok;
        if (act0) {
            ub0 = fast_upper<L, JIT>(st, accf_lane(A, 0), ck, nsum, lgP0, s20, e0, ome0, ec0,
                                     dub, ok);
            h0 = lb_ok && ok && ub0 + dub < lim;
        }
        if (act1) {
            ub1 = fast_upper<L, JIT>(st, accf_lane(A, 1), ck, nsum, lgP1, s21, e1, ome1, ec1,
                                     dub, ok);
            h1 = lb_ok && ok && ub1 + dub < lim;
        }
    }
    return __all_sync(0xffffffffu, h0 && h1);
}

// Resident CTAs per SM the FP32-sum kernel is compiled for: 8 (64 registers,
// 32 warps) measured 1-2 % faster than 7, 6 or 5 on GB300.
#ifndef JOKER_FAST_MINB
#define JOKER_FAST_MINB 8
#endif

// Two samples per thread (paired FP32), any L without jitter, L <= 3 with.
// FUSED: also the first acceptance pass (implicit work items, chunks of at
// most FUSED_MAX_CHUNK samples): each sample's uniform from its slot's PCG64
// stream and its candidate bit.
template <int L, bool JIT, bool PACKED, bool FUSED, bool EXIT = false>
__global__ void __launch_bounds__(128, JOKER_FAST_MINB)
lnl_fast2_kernel(LnlArgs a) {
    static_assert(!EXIT || (FUSED && L <= 3), "early exit is part of the fused pass, L <= 3");
    // the out-of-reach test after the last epoch: always in the fused pass
    // (L <= 3), on request (oor_tail) in the plain form (L <= 3, or 4 without
    // jitter)
    constexpr bool OOR = FUSED ? (L <= 3) : (L <= 3 || (L == 4 && !JIT));
    __shared__ __align__(16) float sm[TILE * REC32];
    __shared__ double smr[PACKED ? PACK_ROWS * 5 : 1];
    __shared__ unsigned long long s_pcg[FUSED ? 2 * FUSED_PASSES + 4 : 1];
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
        if (FUSED && threadIdx.x == 0) fused_item_states(a, w, s_pcg);
        if (single && w.star != staged_star) {
            stage_epochs<float, REC32>(sm, a.ep32 + (size_t)st.epoch_off * REC32, N);
            staged_star = w.star;
            __syncthreads();
        } else if (FUSED) {
            __syncthreads();
        }
        unsigned long long *mk = a.max_key ? a.max_key + w.max_slot : nullptr;
        unsigned long long *bk = a.bound_key ? a.bound_key + 2 * w.max_slot : nullptr;
        for (int base = 0; base < w.count; base += 2 * blockDim.x) {
            const int j0 = base + threadIdx.x, j1 = j0 + blockDim.x;
            const bool act0 = j0 < w.count, act1 = j1 < w.count;
            float4 pa0, pb0, pa1, pb1;
            float s20, s21;
            load_pair<JIT, PACKED>(a, w, base, smr, inter, act0, act1, pa0, pb0, s20, pa1, pb1,
                                   s21);
            const MixC<float> c0 = mix_consts(pa0, pb0, s20), c1 = mix_consts(pa1, pb1, s21);
            const MixC<float2> c = mix_pair(c0, c1);
            AccF<L, JIT, float2> A;
            A.zero();
            bool exited = false;
            float ub0 = 0.0f, ub1 = 0.0f;
            // column-error constant of a sample with 1/P = iph: the empirical
            // part plus the split phase's rounding over the star's span
            auto col_c0 = [&](float iph) { return fmaf(st.phase_c, iph, a.err_c0); };
            // every epoch, staged a tile at a time for long stars
            auto all_epochs = [&]() {
                for (int t0 = 0; t0 < N; t0 += TILE) {
                    const int nt = min(TILE, N - t0);
                    if (!single) {
                        __syncthreads();
                        stage_epochs<float, REC32>(sm, a.ep32 + ((size_t)st.epoch_off + t0) * REC32,
                                                   nt);
                        staged_star = -1;
                        __syncthreads();
                    }
                    if (act0) {
#pragma unroll 2
                        for (int i = 0; i < nt; ++i)
                            fast_epoch<L, JIT, false>(sm + i * REC32, c, A);
                    }
                }
            };
            if constexpr (EXIT) {
                if (single) {
                    // the epochs in segments ending at the star's checkpoints;
                    // the warp stops once all its samples are out of reach
                    int i0 = 0;
                    for (int q = 0; q < st.n_ck; ++q) {
                        const int kend = st.ck_k[q];
                        if (act0) {
#pragma unroll 2
                            for (int i = i0; i < kend; ++i)
                                fast_epoch<L, JIT, false>(sm + i * REC32, c, A);
                        }
                        i0 = kend;
                        if (warp_out_of_reach<L, JIT>(st, A, st.ck[q], kend, c0.e, c0.ome, c1.e,
                                                      c1.ome, pb0.w, pb1.w, s20, s21,
                                                      col_c0(c.iph.x), col_c0(c.iph.y), act0,
                                                      act1, bk, ub0, ub1)) {
                            exited = true;
                            break;
                        }
                    }
                    if (!exited) {
                        if (act0) {
#pragma unroll 2
                            for (int i = i0; i < N; ++i)
                                fast_epoch<L, JIT, false>(sm + i * REC32, c, A);
                        }
                        // all epochs: the same test on the full sums spares the
                        // float-float tail and its bound (ub is then ln L in FP32)
                        exited = warp_out_of_reach<L, JIT>(
                            st, A, st.ck_full, N, c0.e, c0.ome, c1.e, c1.ome, pb0.w, pb1.w, s20,
                            s21, col_c0(c.iph.x), col_c0(c.iph.y), act0, act1, bk, ub0, ub1);
                    }
                } else {
                    all_epochs();
                    exited = warp_out_of_reach<L, JIT>(
                        st, A, st.ck_full, N, c0.e, c0.ome, c1.e, c1.ome, pb0.w, pb1.w, s20, s21,
                        col_c0(c.iph.x), col_c0(c.iph.y), act0, act1, bk, ub0, ub1);
                }
            } else {
                all_epochs();
                if constexpr (OOR) {
                    // every epoch evaluated: a warp whose samples are all out of
                    // reach (rejected for every uniform, not the maximum) keeps
                    // their ln L in FP32 and skips the float-float tail and
                    // bound (the fused pass, or on request)
                    if (FUSED || (a.oor_tail && bk))
                        exited = warp_out_of_reach<L, JIT>(
                            st, A, st.ck_full, N, c0.e, c0.ome, c1.e, c1.ome, pb0.w, pb1.w, s20,
                            s21, col_c0(c.iph.x), col_c0(c.iph.y), act0, act1, bk, ub0, ub1);
                }
            }
            if ((EXIT || OOR) && exited) {
                // ln L of these samples is left at their upper bound (or, after
                // the last epoch, at its FP32 value), with an infinite error
                // bound; they carry no candidate bit and no key
                if (act0) {
                    a.lnl[w.out_off + j0] = (double)ub0;
                    a.err[w.out_off + j0] = __int_as_float(0x7f800000);
                }
                if (act1) {
                    a.lnl[w.out_off + j1] = (double)ub1;
                    a.err[w.out_off + j1] = __int_as_float(0x7f800000);
                }
                if constexpr (FUSED) fused_write_words(a, w, base, 0u, 0u);
                continue;
            }
            ff l0 = ffv(0.0f), l1 = ffv(0.0f);
            float err0 = 0.0f, err1 = 0.0f;
            if (act0)
                fast_tail<L, JIT>(st, accf_lane(A, 0), c0.e, c0.ome, pb0.w, s20, N,
                                  col_c0(c.iph.x), l0, err0);
            if (act1)
                fast_tail<L, JIT>(st, accf_lane(A, 1), c1.e, c1.ome, pb1.w, s21, N,
                                  col_c0(c.iph.y), l1, err1);
            const unsigned long long kd =
                fast_store2(a, w.out_off + j0, act0, l0, err0, w.out_off + j1, act1, l1, err1, mk,
                            bk);
            fused_pass<FUSED>(a, w, base, s_pcg, kd, bk, act0, l0, err0, act1, l1, err1);
        }
    }
}

// Launch over the kernel's forms: the prepared cache, or packed FP64 rows
// prepared in registers (cache views); L <= 6 without the jitter, L <= 3
// with it.
template <bool FUSED, int L, bool JIT>
static cudaError_t launch_fast_LJ(const LnlArgs &a, int block, cudaStream_t st) {
    if constexpr (FUSED && L <= 3) {
        if (a.fa_exit) {
            if (a.mx_a == nullptr)
                return launch_persistent(lnl_fast2_kernel<L, JIT, true, true, true>, a, block, st);
            return launch_persistent(lnl_fast2_kernel<L, JIT, false, true, true>, a, block, st);
        }
    }
    if (a.mx_a == nullptr)
        return launch_persistent(lnl_fast2_kernel<L, JIT, true, FUSED>, a, block, st);
    return launch_persistent(lnl_fast2_kernel<L, JIT, false, FUSED>, a, block, st);
}

template <bool FUSED>
cudaError_t launch_fast_any(int L, bool jit, const LnlArgs &a, int block, cudaStream_t st) {
    if (jit) {
        switch (L) {
            case 1: return launch_fast_LJ<FUSED, 1, true>(a, block, st);
            case 2: return launch_fast_LJ<FUSED, 2, true>(a, block, st);
            case 3: return launch_fast_LJ<FUSED, 3, true>(a, block, st);
        }
        return cudaErrorInvalidValue;
    }
    switch (L) {
        case 1: return launch_fast_LJ<FUSED, 1, false>(a, block, st);
        case 2: return launch_fast_LJ<FUSED, 2, false>(a, block, st);
        case 3: return launch_fast_LJ<FUSED, 3, false>(a, block, st);
        case 4: return launch_fast_LJ<FUSED, 4, false>(a, block, st);
        case 5: return launch_fast_LJ<FUSED, 5, false>(a, block, st);
        case 6: return launch_fast_LJ<FUSED, 6, false>(a, block, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace joker
