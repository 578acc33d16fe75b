// FP64 per-sample marginal likelihood, shared by the FP64 kernel and the
// refinement step of the acceptance pass (both must give identical numbers).
#pragma once
#include "joker_internal.cuh"
#include "joker_math.cuh"

namespace joker {

// Natural log of a positive double for the FP64-tail variant of the mixed
// path: exact binary exponent, FP32 logf of the mantissa in [1, 2).
__device__ __forceinline__ double log_mixed(double x) {
    const int hi = __double2hiint(x);
    const int ex = ((hi >> 20) & 0x7ff) - 1023;
    const double m = __hiloint2double((hi & 0x800fffff) | 0x3ff00000, __double2loint(x));
    if (ex == -1023 || ex == 1024) return log(x);   // zero, subnormal, inf, NaN
    return (double)ex * 0.69314718055994530942 + (double)logf((float)m);
}

// One Keplerian orbit in FP64: the unit-K radial velocity
//   m(dt) = cos(omega + f) + e cos(omega),  M = 2 pi dt / P - M0,
// in terms of the eccentric anomaly, m = (A cos E + B sin E - D)/(1 - e cos E) + D
// with A = cos omega, B = -sin omega sqrt(1 - e^2), D = e cos omega (the model
// twobody's c_rv_from_elements evaluates for thejoker/src/fast_likelihood.pyx
// :453-455).
struct OrbitF64 {
    double e, Ac, Bc, Dc, k2p, M0;
    float ef, omef, a1f;                 // the Kepler solver's FP32 constants

    __device__ __forceinline__ void init(double P, double e_, double om, double M0_) {
        e = e_;
        M0 = M0_;
        k2p = TWO_PI_D / P;                  // correctly rounded: it scales every phase
        double sw, cw;
        sincos_f64_table(om, sw, cw);
        Ac = cw;
        Bc = -sw * sqrt((1.0 - e) * (1.0 + e));
        Dc = e * cw;
        kepler_consts_f32(e, ef, omef, a1f);
    }

    __device__ __forceinline__ double rv_unit(double dt) const {
        double M = fma(dt, k2p, -M0);
        const double nrev = rint(M * INV_TWO_PI_D);
        M = fma(-nrev, TWO_PI_HI_D, M);
        M = fma(-nrev, TWO_PI_LO_D, M);
        double sE, cE;
        kepler_sincos_f64(M, e, ef, omef, a1f, sE, cE);
        return fma(fma(Ac, cE, fma(Bc, sE, -Dc)), rcp_newton(fma(-e, cE, 1.0)), Dc);
    }
};

// Per-sample FP64 state: the epoch sums and the sample's constants.
template <int L, bool JIT>
struct Acc64 {
    OrbitF64 orb;
    double s2, mu0;
    double A00, b0, A0[MAXL];            // no jitter
    double G[L][L], q[L], rWr;           // jitter: full system
    // jitter: prod_j (1 + s^2 ivar_j) = pj 2^ej (pj in [1, 2) after each
    // epoch) plus slog, the logs already summed (warp_sum); sum log w_j is
    // sum log ivar_j - log of the product.
    double pj, slog;
    int ej;

    __device__ __forceinline__ void init(const StarRec &st, double P, double e_, double om,
                                         double M0_, double s_) {
        orb.init(P, e_, om, M0_);
        s2 = s_ * s_;
        mu0 = st.mu0;
        A00 = 0.0;
        b0 = 0.0;
#pragma unroll
        for (int k = 0; k < MAXL; ++k) A0[k] = 0.0;
        rWr = 0.0;
        pj = 1.0;
        slog = 0.0;
        ej = 0;
        if (JIT) {
#pragma unroll
            for (int i = 0; i < L; ++i) {
                q[i] = 0.0;
#pragma unroll
                for (int k = 0; k < L; ++k) G[i][k] = 0.0;
            }
        }
    }

    // one epoch: dt = t - t_ref, y' = y - sum_{j>=1} mu_j T_j, ivar, T_1..T_{L-1}
    __device__ __forceinline__ void add(double dt, double yp, double iv, const double *T) {
        const double m = orb.rv_unit(dt);
        if (!JIT) {
            const double wm = iv * m;
            A00 = fma(wm, m, A00);
            b0 = fma(wm, yp, b0);
#pragma unroll
            for (int k = 1; k < L; ++k) A0[k] = fma(wm, T[k - 1], A0[k]);
        } else {
            const double dj = fma(s2, iv, 1.0);
            const double wj = iv * rcp_newton(dj);
            // pj *= dj, then the binary exponent moves to ej (integer ops);
            // dj >= 1 keeps pj >= 1, a positive normal number
            pj *= dj;
            const int hi = __double2hiint(pj);
            ej += (hi >> 20) - 1023;
            pj = __hiloint2double((hi & 0x000fffff) | 0x3ff00000, __double2loint(pj));
            double x[L];
            x[0] = m;
#pragma unroll
            for (int k = 1; k < L; ++k) x[k] = T[k - 1];
            const double r = fma(-mu0, m, yp);
            rWr = fma(wj * r, r, rWr);
#pragma unroll
            for (int ii = 0; ii < L; ++ii) {
                const double wx = wj * x[ii];
                q[ii] = fma(wx, r, q[ii]);
#pragma unroll
                for (int k = 0; k <= ii; ++k) G[ii][k] = fma(wx, x[k], G[ii][k]);
            }
        }
    }

    // Sum the epoch sums of the 32 lanes of a warp (every lane gets the total).
    __device__ __forceinline__ void warp_sum() {
        if (!JIT) {
            A00 = wsum(A00);
            b0 = wsum(b0);
#pragma unroll
            for (int k = 1; k < L; ++k) A0[k] = wsum(A0[k]);
        } else {
            rWr = wsum(rWr);
            slog = wsum(log_prod());
            pj = 1.0;
            ej = 0;
#pragma unroll
            for (int ii = 0; ii < L; ++ii) {
                q[ii] = wsum(q[ii]);
#pragma unroll
                for (int k = 0; k <= ii; ++k) G[ii][k] = wsum(G[ii][k]);
            }
        }
    }

    // sum_j log(1 + s^2 ivar_j) over the epochs this accumulator has seen
    __device__ __forceinline__ double log_prod() const {
        return fma((double)ej, 0.69314718055994530942, slog + log(pj));
    }

    // sum_j log w_j, w_j = ivar_j / (1 + s^2 ivar_j)
    __device__ __forceinline__ double sum_log_w(const StarRec &st) const {
        return st.sum_log_ivar - log_prod();
    }

    static __device__ __forceinline__ double wsum(double x) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        return x;
    }

    __device__ __forceinline__ double finish(const StarRec &st, double P) const;
};

// Schur-complement tail (no jitter), FP64.
template <int L, bool MIXED_LOG>
__device__ __forceinline__ double tail_schur_d(const StarRec &st, double A00, const double *A0,
                                               double b0, double lam0, double log_lam0) {
    double gv = 0.0, gcC = 0.0;
#pragma unroll
    for (int j = 1; j < L; ++j) {
        double vj = 0.0;
#pragma unroll
        for (int k = 1; k < L; ++k) vj = fma(st.Cinv[j * MAXL + k], A0[k], vj);
        gv = fma(A0[j], vj, gv);
        gcC = fma(A0[j], st.cC[j], gcC);
    }
    const double a_minus = A00 - gv;           // s - 1/Lambda0
    const double u = b0 - gcC;
    const double mu0 = st.mu0;
    const double t = fma(-mu0, a_minus, u);
    double chi2 = st.chi2_0;
    if (mu0 != 0.0) chi2 = fma(mu0 * mu0, a_minus, fma(-2.0 * mu0, u, chi2));
    if constexpr (MIXED_LOG) {
        const double s = a_minus + 1.0 / lam0;
        chi2 -= t * t / s;
        return -0.5 * (chi2 + st.logdet_const + log_lam0 + log_mixed(s));
    } else {
        // Lambda0 s = Lambda0 (s - 1/Lambda0) + 1: t^2 / s and log Lambda0 + log s
        // from one reciprocal and one log
        const double ls = fma(lam0, a_minus, 1.0);
        chi2 = fma(-t * t * lam0, rcp_newton(ls), chi2);
        return -0.5 * (chi2 + st.logdet_const + log(ls));
    }
}

// Full tail (jitter applied), FP64: LDL^T of G, quadratic form, log det.
// logdet_const + log(scale * det G) is the log-determinant term.
template <int L, bool MIXED_LOG>
__device__ __forceinline__ double tail_full_d(const double (&G)[L][L], const double (&q)[L],
                                              double rWr, double logdet_const,
                                              double scale = 1.0) {
    double D[L], rD[L], Lw[L][L];
    double quad = 0.0, detp = 1.0;
#pragma unroll
    for (int k = 0; k < L; ++k) {
        double dk = G[k][k];
#pragma unroll
        for (int m = 0; m < k; ++m) dk = fma(-Lw[k][m] * Lw[k][m], D[m], dk);
        D[k] = dk;
        const double rdk = rcp_newton(dk);
        rD[k] = rdk;
#pragma unroll
        for (int i = k + 1; i < L; ++i) {
            double v = G[i][k];
#pragma unroll
            for (int m = 0; m < k; ++m) v = fma(-Lw[i][m] * Lw[k][m], D[m], v);
            Lw[i][k] = v * rdk;
        }
        detp *= dk;
    }
    double z[L];
#pragma unroll
    for (int k = 0; k < L; ++k) {
        double v = q[k];
#pragma unroll
        for (int m = 0; m < k; ++m) v = fma(-Lw[k][m], z[m], v);
        z[k] = v;
        quad = fma(v * v, rD[k], quad);
    }
    const double logdet = logdet_const + (MIXED_LOG ? log_mixed(detp) : log(scale * detp));
    return -0.5 * (rWr - quad + logdet);
}

// K prior variance per sample (fast_likelihood.pyx:461-464)
__device__ __forceinline__ double k_prior_variance(const StarRec &st, double P, double e) {
    if (!st.k_scaled) return st.lam0;
    const double y = rcbrt_newton(P * st.iP0);                  // (P / P0)^(-1/3)
    const double v = st.sigK0sq * (y * y) * rcp_newton(1.0 - e * e);
    return fmin(st.maxK2, v);
}

template <int L, bool JIT>
__device__ __forceinline__ double Acc64<L, JIT>::finish(const StarRec &st, double P) const {
    const double lam0 = k_prior_variance(st, P, orb.e);
    if constexpr (!JIT) {
        return tail_schur_d<L, false>(st, A00, A0, b0, lam0, 0.0);
    } else {
        double Gs[L][L];
        const double ilam0 = st.k_scaled ? rcp_newton(lam0) : st.ilam[0];
#pragma unroll
        for (int ii = 0; ii < L; ++ii) {
#pragma unroll
            for (int k = 0; k <= ii; ++k) { Gs[ii][k] = G[ii][k]; Gs[k][ii] = G[ii][k]; }
            Gs[ii][ii] += ii == 0 ? ilam0 : st.ilam[ii];
        }
        // log det term: log_norm_rest + log Lambda0 - sum log w + log det G, with
        // -sum log w = -sum log ivar + slog + ej ln 2 + log pj
        return tail_full_d<L, false>(
            Gs, q, rWr,
            fma((double)ej, 0.69314718055994530942, st.log_norm_rest - st.sum_log_ivar + slog),
            lam0 * pj);
    }
}

// FP64 ln L of one sample with the star's epochs read from global memory.
template <int L, bool JIT>
__device__ __noinline__ double fp64_lnl_global(const StarRec &st, const double *ep64, double P,
                                               double e, double om, double M0, double s) {
    Acc64<L, JIT> acc;
    acc.init(st, P, e, om, M0, s);
    const double *rec = ep64 + (size_t)st.epoch_off * REC64;
    for (int i = 0; i < st.n_epochs; ++i, rec += REC64) {
        double T[MAXL];
#pragma unroll
        for (int k = 1; k < L; ++k) T[k - 1] = __ldg(rec + 2 + k);
        acc.add(__ldg(rec), __ldg(rec + 1), __ldg(rec + 2), T);
    }
    return acc.finish(st, P);
}

// FP64 ln L of one sample evaluated by a whole warp: lane l takes epochs l,
// l + 32, ...; the sums are combined across the warp.  All 32 lanes must call
// it with the same sample; all return the value.  Same arithmetic per epoch
// as fp64_lnl_global, summed in a different order (agreement to FP64
// rounding of the sums).
template <int L, bool JIT>
__device__ __noinline__ double fp64_lnl_warp_t(const StarRec &st, const double *ep64, double P,
                                               double e, double om, double M0, double s) {
    Acc64<L, JIT> acc;
    acc.init(st, P, e, om, M0, s);
    const double *rec0 = ep64 + (size_t)st.epoch_off * REC64;
    for (int i = threadIdx.x & 31; i < st.n_epochs; i += 32) {
        const double *rec = rec0 + (size_t)i * REC64;
        double T[MAXL];
#pragma unroll
        for (int k = 1; k < L; ++k) T[k - 1] = __ldg(rec + 2 + k);
        acc.add(__ldg(rec), __ldg(rec + 1), __ldg(rec + 2), T);
    }
    acc.warp_sum();
    return acc.finish(st, P);
}

__device__ __forceinline__ double fp64_lnl_warp(int L, bool jit, const StarRec &st,
                                                const double *ep64, double P, double e,
                                                double om, double M0, double s) {
    switch (L) {
        case 1: return jit ? fp64_lnl_warp_t<1, true>(st, ep64, P, e, om, M0, s)
                           : fp64_lnl_warp_t<1, false>(st, ep64, P, e, om, M0, s);
        case 2: return jit ? fp64_lnl_warp_t<2, true>(st, ep64, P, e, om, M0, s)
                           : fp64_lnl_warp_t<2, false>(st, ep64, P, e, om, M0, s);
        case 3: return jit ? fp64_lnl_warp_t<3, true>(st, ep64, P, e, om, M0, s)
                           : fp64_lnl_warp_t<3, false>(st, ep64, P, e, om, M0, s);
        case 4: return jit ? fp64_lnl_warp_t<4, true>(st, ep64, P, e, om, M0, s)
                           : fp64_lnl_warp_t<4, false>(st, ep64, P, e, om, M0, s);
        case 5: return jit ? fp64_lnl_warp_t<5, true>(st, ep64, P, e, om, M0, s)
                           : fp64_lnl_warp_t<5, false>(st, ep64, P, e, om, M0, s);
        default: return jit ? fp64_lnl_warp_t<6, true>(st, ep64, P, e, om, M0, s)
                            : fp64_lnl_warp_t<6, false>(st, ep64, P, e, om, M0, s);
    }
}

__device__ __forceinline__ double fp64_lnl_sample(int L, bool jit, const StarRec &st,
                                                  const double *ep64, double P, double e,
                                                  double om, double M0, double s) {
    switch (L) {
        case 1: return jit ? fp64_lnl_global<1, true>(st, ep64, P, e, om, M0, s)
                           : fp64_lnl_global<1, false>(st, ep64, P, e, om, M0, s);
        case 2: return jit ? fp64_lnl_global<2, true>(st, ep64, P, e, om, M0, s)
                           : fp64_lnl_global<2, false>(st, ep64, P, e, om, M0, s);
        case 3: return jit ? fp64_lnl_global<3, true>(st, ep64, P, e, om, M0, s)
                           : fp64_lnl_global<3, false>(st, ep64, P, e, om, M0, s);
        case 4: return jit ? fp64_lnl_global<4, true>(st, ep64, P, e, om, M0, s)
                           : fp64_lnl_global<4, false>(st, ep64, P, e, om, M0, s);
        case 5: return jit ? fp64_lnl_global<5, true>(st, ep64, P, e, om, M0, s)
                           : fp64_lnl_global<5, false>(st, ep64, P, e, om, M0, s);
        default: return jit ? fp64_lnl_global<6, true>(st, ep64, P, e, om, M0, s)
                            : fp64_lnl_global<6, false>(st, ep64, P, e, om, M0, s);
    }
}

}  // namespace joker
