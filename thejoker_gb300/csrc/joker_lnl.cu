// Marginal-likelihood kernels of libjoker_gb300 (sm_103a).
//
// Both kernels evaluate, for one star and one prior sample (P, e, omega, M0, s),
// the ln-likelihood with the linear parameters (K, v0, offsets, trend)
// integrated out under their Gaussian prior -- the quantity the reference
// computes in CJokerHelper.likelihood_worker (thejoker/src/fast_likelihood.pyx
// :359-425) through an N x N LU factorisation.  Here the same number comes
// from the matrix determinant lemma and the Woodbury identity in O(N L^2):
//
//   G = Lambda^-1 + M W M^T (L x L),  q = M W r,  r = y - M^T mu
//   chi2   = r^T W r - q^T G^-1 q
//   logdet = N log(2 pi) - sum log w + sum log Lambda_i + log det G
//   ln L   = -(chi2 + logdet) / 2
//
// Row 0 of M is the unit-K Kepler velocity, rows 1.. the trend/offset
// columns.  Everything that does not depend on the sample (the trend block of
// G, its inverse, the trend-only chi2) is folded per star on the host, so per
// sample only the Schur complement s = G00 - g^T C^-1 g and one scalar
// quadratic remain:  chi2 = chi2_0 - 2 mu0 u + mu0^2 (s - 1/Lambda0) - t^2 / s,
// u = b0 - g^T C^-1 c,  t = u - mu0 (s - 1/Lambda0).
//
// One thread owns one sample and walks the star's epochs, which the CTA
// stages in shared memory; CTAs pull (star, sample-range) work items from a
// global counter (a persistent launch sized to the SM count).
#include "joker_internal.cuh"
#include "joker_math.cuh"

namespace joker {

// ------------------------------------------------------------------ staging
template <typename T, int REC>
__device__ __forceinline__ void stage_epochs(T *sm, const T *src, int n) {
    // n records of REC elements, copied with 16-byte vectors
    const int nvec = n * REC * (int)sizeof(T) / 16;
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
    float4 *d4 = reinterpret_cast<float4 *>(sm);
    for (int i = threadIdx.x; i < nvec; i += blockDim.x) d4[i] = __ldg(s4 + i);
}

// Natural log of a positive double for the mixed path: the binary exponent is
// taken exactly and only the mantissa in [1, 2) goes through FP32 logf, so the
// absolute error stays near 1e-7 at any magnitude.
__device__ __forceinline__ double log_mixed(double x) {
    const int hi = __double2hiint(x);
    const int ex = ((hi >> 20) & 0x7ff) - 1023;
    const double m = __hiloint2double((hi & 0x800fffff) | 0x3ff00000, __double2loint(x));
    if (ex == -1023 || ex == 1024) return log(x);   // zero, subnormal, inf, NaN
    return (double)ex * 0.69314718055994530942 + (double)logf((float)m);
}

// Warp-aggregated update of the running maximum of one star.
__device__ __forceinline__ void update_max(unsigned long long *max_key, double v, bool active) {
    if (max_key == nullptr) return;
    unsigned long long k = active ? double_to_key(v) : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long other = __shfl_xor_sync(0xffffffffu, k, o);
        k = other > k ? other : k;
    }
    if ((threadIdx.x & 31) == 0 && k != 0ull) {
        if (k > *((volatile unsigned long long *)max_key)) atomicMax(max_key, k);
    }
}

// Per-sample tail shared by both kernels (FP64): from the epoch sums
// A00 = sum w m^2, A0j = sum w m T_j, b0 = sum w m y' and the star constants.
template <int L, bool MIXED_LOG>
__device__ __forceinline__ double lnl_tail_nojitter(const StarRec &st, double A00,
                                                    const double *A0, double b0,
                                                    double lam0, double log_lam0) {
    // v = C^-1 g over the trend block (rows/cols 1..L-1)
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
    const double s = a_minus + 1.0 / lam0;
    const double u = b0 - gcC;
    const double mu0 = st.mu0;
    const double t = fma(-mu0, a_minus, u);
    double chi2 = st.chi2_0;
    if (mu0 != 0.0) chi2 = fma(mu0 * mu0, a_minus, fma(-2.0 * mu0, u, chi2));
    chi2 -= t * t / s;
    const double logdet = st.logdet_const + log_lam0 + (MIXED_LOG ? log_mixed(s) : log(s));
    return -0.5 * (chi2 + logdet);
}

// General tail (jitter applied): full L x L system, LDL^T factorisation.
template <int L, bool MIXED_LOG>
__device__ __forceinline__ double lnl_tail_full(const double (&G)[L][L], const double (&q)[L],
                                                double rWr, double logdet_const) {
    double D[L], Lw[L][L];
    double logdet = logdet_const, quad = 0.0, detp = 1.0;
#pragma unroll
    for (int k = 0; k < L; ++k) {
        double dk = G[k][k];
#pragma unroll
        for (int m = 0; m < k; ++m) dk = fma(-Lw[k][m] * Lw[k][m], D[m], dk);
        D[k] = dk;
        const double rdk = 1.0 / dk;
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
        quad = fma(v * v, 1.0 / D[k], quad);
    }
    logdet += (MIXED_LOG ? log_mixed(detp) : log(detp));
    return -0.5 * (rWr - quad + logdet);
}

// ------------------------------------------------------------- K1: FP64 path
// Epoch record (REC64 doubles): dt, y', ivar, T_1..T_{L-1}.
template <int L, bool JIT>
__global__ void __launch_bounds__(128)
lnl_fp64_kernel(LnlArgs a) {
    __shared__ __align__(16) double sm[TILE * REC64];
    __shared__ int s_item;
    int staged_star = -1;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.queue, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= a.n_items) break;
        const WorkItem w = get_item(a, it);
        const StarRec &st = a.stars[w.star];
        const int N = st.n_epochs;
        const bool single = N <= TILE;
        if (single && w.star != staged_star) {
            stage_epochs<double, REC64>(sm, a.ep64 + (size_t)st.epoch_off * REC64, N);
            staged_star = w.star;
            __syncthreads();
        }
        unsigned long long *mk = a.max_key ? a.max_key + w.max_slot : nullptr;
        for (int base = 0; base < w.count; base += blockDim.x) {
            const int j = base + threadIdx.x;
            const bool active = j < w.count;
            const int64_t row = w.row0 + (active ? j : 0);
            const double P = a.P[row * a.stride], e = a.e[row * a.stride];
            const double om = a.om[row * a.stride], M0 = a.M0[row * a.stride];
            const double sj = JIT ? a.s[row * a.stride] : 0.0;
            const double k2p = TWO_PI_D / P;
            double sw, cw;
            sincos(om, &sw, &cw);
            const double sq1me2 = sqrt((1.0 - e) * (1.0 + e));
            const double Ac = cw, Bc = -sw * sq1me2, Dc = e * cw;
            // K prior variance (fast_likelihood.pyx:461-464)
            double lam0;
            if (st.k_scaled) {
                const double v = st.sigK0sq / (1.0 - e * e) * pow(P / st.P0, -2.0 / 3.0);
                lam0 = fmin(st.maxK2, v);
            } else {
                lam0 = st.lam0;
            }
            double A00 = 0.0, b0 = 0.0, A0[MAXL];
#pragma unroll
            for (int k = 0; k < MAXL; ++k) A0[k] = 0.0;
            // jitter-applied sums (full system)
            double G[L][L], q[L], rWr = 0.0, slw = 0.0;
            if (JIT) {
#pragma unroll
                for (int i = 0; i < L; ++i) {
                    q[i] = 0.0;
#pragma unroll
                    for (int k = 0; k < L; ++k) G[i][k] = 0.0;
                }
            }
            for (int t0 = 0; t0 < N; t0 += TILE) {
                const int nt = min(TILE, N - t0);
                if (!single) {
                    __syncthreads();
                    stage_epochs<double, REC64>(sm, a.ep64 + ((size_t)st.epoch_off + t0) * REC64, nt);
                    __syncthreads();
                }
                if (active) {
                    for (int i = 0; i < nt; ++i) {
                        const double *rec = sm + i * REC64;
                        const double dt = rec[0], yp = rec[1], iv = rec[2];
                        double M = fma(dt, k2p, -M0);
                        const double nrev = rint(M * INV_TWO_PI_D);
                        M = fma(-nrev, TWO_PI_HI_D, M);
                        M = fma(-nrev, TWO_PI_LO_D, M);
                        double sE, cE;
                        kepler_sincos_f64(M, e, sE, cE);
                        const double den = 1.0 - e * cE;
                        const double m = fma(Ac, cE, fma(Bc, sE, -Dc)) / den + Dc;
                        if (!JIT) {
                            const double wm = iv * m;
                            A00 = fma(wm, m, A00);
                            b0 = fma(wm, yp, b0);
#pragma unroll
                            for (int k = 1; k < L; ++k) A0[k] = fma(wm, rec[2 + k], A0[k]);
                        } else {
                            const double wj = iv / (1.0 + sj * sj * iv);
                            slw += log(wj);
                            double x[L];
                            x[0] = m;
#pragma unroll
                            for (int k = 1; k < L; ++k) x[k] = rec[2 + k];
                            // r = y' - mu0 m
                            const double r = fma(-st.mu0, m, yp);
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
                }
            }
            double lnl = 0.0;
            if (active) {
                if (!JIT) {
                    lnl = lnl_tail_nojitter<L, false>(st, A00, A0, b0, lam0, log(lam0));
                } else {
#pragma unroll
                    for (int ii = 0; ii < L; ++ii) {
                        G[ii][ii] += 1.0 / (ii == 0 ? lam0 : st.lam[ii]);
#pragma unroll
                        for (int k = ii + 1; k < L; ++k) G[ii][k] = G[k][ii];
                    }
                    lnl = lnl_tail_full<L, false>(G, q, rWr, st.log_norm_rest + log(lam0) - slw);
                }
                a.lnl[w.out_off + j] = lnl;
            }
            update_max(mk, lnl, active);
        }
    }
}

// ----------------------------------------------------------- K2: mixed path
// Epoch record (REC32 floats), no jitter:
//   dt_hi, dt_lo, w_hi, w_lo, wy_hi, wy_lo, (wT_j hi, lo) for j = 1..L-1
// with jitter:
//   dt_hi, dt_lo, ivar, 0, y_hi, y_lo, (T_j hi, lo) for j = 1..L-1
// Phase: frac(dt / P - M0 / 2 pi) in float-float (exact to ~2^-46 of the
// cycle count), rounded once to FP32.  Kepler and the velocity column in
// FP32; every epoch sum in float-float with exact products; the per-sample
// tail in FP64.
template <int L, bool JIT, bool ACC_SINCOS>
__global__ void __launch_bounds__(128)
lnl_mixed_kernel(LnlArgs a) {
    __shared__ __align__(16) float sm[TILE * REC32];
    __shared__ int s_item;
    int staged_star = -1;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.queue, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= a.n_items) break;
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
        for (int base = 0; base < w.count; base += blockDim.x) {
            const int j = base + threadIdx.x;
            const bool active = j < w.count;
            const int64_t row = w.row0 + (active ? j : 0);
            const float4 pa = __ldg(a.mx_a + row);
            const float4 pb = __ldg(a.mx_b + row);
            const float s2 = JIT ? __ldg(a.mx_s2 + row) : 0.0f;
            const float e = pb.x, ome = 1.0f - e;
            const float a1 = (float)MK_A1_D * fast_rcp(1.0f + e);
            const float sq1me2 = sqrtf(ome * (1.0f + e));
            const float Ac = pb.y, Bc = -pb.z * sq1me2, Dc = e * pb.y;
            // accumulators (float-float)
            float A00h = 0.f, A00l = 0.f, bh = 0.f, bl = 0.f;
            float Ah[MAXL], Al[MAXL];
#pragma unroll
            for (int k = 0; k < MAXL; ++k) { Ah[k] = 0.f; Al[k] = 0.f; }
            // jitter: full Gram matrix, q, r^T W r, sum log2(1 + s^2 ivar)
            float Gh[L][L], Gl[L][L], qh[L], ql[L], rh = 0.f, rl = 0.f, lg2 = 0.f;
            if (JIT) {
#pragma unroll
                for (int i = 0; i < L; ++i) {
                    qh[i] = ql[i] = 0.f;
#pragma unroll
                    for (int k = 0; k < L; ++k) Gh[i][k] = Gl[i][k] = 0.f;
                }
            }
            for (int t0 = 0; t0 < N; t0 += TILE) {
                const int nt = min(TILE, N - t0);
                if (!single) {
                    __syncthreads();
                    stage_epochs<float, REC32>(sm, a.ep32 + ((size_t)st.epoch_off + t0) * REC32, nt);
                    __syncthreads();
                }
                if (active) {
#pragma unroll 2
                    for (int i = 0; i < nt; ++i) {
                        const float *rec = sm + i * REC32;
                        const float4 r0 = *reinterpret_cast<const float4 *>(rec);
                        // ---- phase in cycles: dt * (1/P) - M0/(2 pi), mod 1
                        const float p = __fmul_rn(r0.x, pa.x);
                        float pe = __fmaf_rn(r0.x, pa.x, -p);
                        pe = __fmaf_rn(r0.x, pa.y, pe);
                        pe = __fmaf_rn(r0.y, pa.x, pe);
                        const float fr = __fsub_rn(p, rintf(p));         // exact
                        float s1, e1;
                        two_sum(fr, -pa.z, s1, e1);                       // exact
                        const float lo = __fadd_rn(__fadd_rn(pe, e1), -pa.w);
                        const float k = rintf(__fadd_rn(s1, lo));
                        const float f = __fadd_rn(__fsub_rn(s1, k), lo);  // [-0.5, 0.5]
                        const float M = __fmaf_rn(f, TWO_PI_HI_F, f * TWO_PI_LO_F);
                        // ---- Kepler + unit-K velocity
                        float sE, cE;
                        kepler_sincos_f32<ACC_SINCOS>(M, e, ome, a1, sE, cE);
                        const float den = __fmaf_rn(-e, cE, 1.0f);
                        float rd = fast_rcp(den);
                        rd = rd * __fmaf_rn(-den, rd, 2.0f);
                        const float m = __fmaf_rn(__fmaf_rn(Ac, cE, __fmaf_rn(Bc, sE, -Dc)), rd, Dc);
                        if (!JIT) {
                            const float4 r1 = *reinterpret_cast<const float4 *>(rec + 4);
                            // t = w m exactly (two terms)
                            float th, tl;
                            two_prod(r0.z, m, th, tl);
                            tl = __fmaf_rn(r0.w, m, tl);
                            ff_acc(A00h, A00l, th, tl, m);
                            ff_acc(bh, bl, r1.x, r1.y, m);
                            if (L > 1) ff_acc(Ah[1], Al[1], r1.z, r1.w, m);
#pragma unroll
                            for (int kk = 2; kk < L; ++kk)
                                ff_acc(Ah[kk], Al[kk], rec[4 + 2 * kk], rec[5 + 2 * kk], m);
                        } else {
                            const float iv = r0.z;
                            const float onep = __fmaf_rn(s2, iv, 1.0f);
                            const float wj = iv * fast_rcp(onep) ;   // the weight used consistently below
                            lg2 += __log2f(onep);
                            const float4 r1 = *reinterpret_cast<const float4 *>(rec + 4);
                            // x = (m, T_1, ...), each as (hi, lo); y' as (hi, lo)
                            float xh[L], xl[L];
                            xh[0] = m; xl[0] = 0.f;
#pragma unroll
                            for (int kk = 1; kk < L; ++kk) { xh[kk] = rec[4 + 2 * kk]; xl[kk] = rec[5 + 2 * kk]; }
                            // r = y' - mu0 m  (float-float)
                            float rrh, rrl;
                            two_prod(-(float)st.mu0, m, rrh, rrl);
                            {
                                float s_, e_;
                                two_sum(r1.x, rrh, s_, e_);
                                rrl = __fadd_rn(__fadd_rn(rrl, e_), r1.y);
                                rrh = s_;
                            }
                            // wr = w * r (float-float)
                            float wrh, wrl;
                            two_prod(wj, rrh, wrh, wrl);
                            wrl = __fmaf_rn(wj, rrl, wrl);
                            // rWr += wr * r ; q_i += wr * x_i
                            {
                                const float p1 = __fmul_rn(wrh, rrh);
                                float pe1 = __fmaf_rn(wrh, rrh, -p1);
                                pe1 = __fmaf_rn(wrh, rrl, __fmaf_rn(wrl, rrh, pe1));
                                ff_add(rh, rl, p1, pe1);
                            }
#pragma unroll
                            for (int ii = 0; ii < L; ++ii) {
                                const float p1 = __fmul_rn(wrh, xh[ii]);
                                float pe1 = __fmaf_rn(wrh, xh[ii], -p1);
                                pe1 = __fmaf_rn(wrh, xl[ii], __fmaf_rn(wrl, xh[ii], pe1));
                                ff_add(qh[ii], ql[ii], p1, pe1);
                                // w x_i (float-float)
                                float wxh, wxl;
                                two_prod(wj, xh[ii], wxh, wxl);
                                wxl = __fmaf_rn(wj, xl[ii], wxl);
#pragma unroll
                                for (int kk = 0; kk <= ii; ++kk) {
                                    const float p2 = __fmul_rn(wxh, xh[kk]);
                                    float pe2 = __fmaf_rn(wxh, xh[kk], -p2);
                                    pe2 = __fmaf_rn(wxh, xl[kk], __fmaf_rn(wxl, xh[kk], pe2));
                                    ff_add(Gh[ii][kk], Gl[ii][kk], p2, pe2);
                                }
                            }
                        }
                    }
                }
            }
            double lnl = 0.0;
            if (active) {
                // K prior variance in log form: log Lambda0 (FP32 is ample here)
                double log_lam0, lam0;
                if (st.k_scaled) {
                    log_lam0 = fmin(st.log_maxK2, st.log_kscale + (double)pb.w);
                    lam0 = (double)expf((float)log_lam0);
                } else {
                    lam0 = st.lam0;
                    log_lam0 = log(lam0);
                }
                if (!JIT) {
                    double A0d[MAXL];
#pragma unroll
                    for (int kk = 0; kk < MAXL; ++kk) A0d[kk] = ff_to_double(Ah[kk], Al[kk]);
                    lnl = lnl_tail_nojitter<L, true>(st, ff_to_double(A00h, A00l), A0d,
                                               ff_to_double(bh, bl), lam0, log_lam0);
                } else {
                    double G[L][L], q[L];
#pragma unroll
                    for (int ii = 0; ii < L; ++ii) {
                        q[ii] = ff_to_double(qh[ii], ql[ii]);
#pragma unroll
                        for (int kk = 0; kk <= ii; ++kk) {
                            G[ii][kk] = ff_to_double(Gh[ii][kk], Gl[ii][kk]);
                            G[kk][ii] = G[ii][kk];
                        }
                        G[ii][ii] += 1.0 / (ii == 0 ? lam0 : st.lam[ii]);
                    }
                    // sum log w = sum log ivar - ln2 * sum log2(1 + s^2 ivar)
                    const double slw = st.sum_log_ivar - 0.6931471805599453 * (double)lg2;
                    lnl = lnl_tail_full<L, true>(G, q, ff_to_double(rh, rl),
                                                     st.log_norm_rest + log_lam0 - slw);
                }
                a.lnl[w.out_off + j] = lnl;
            }
            update_max(mk, lnl, active);
        }
    }
}

// --------------------------------------------------------- cache preparation
// From the reference's packed chunk (n x 5 row-major FP64: P, e, omega, M0, s)
// to FP64 columns and the prepared mixed form.
__global__ void prepare_cache_kernel(const double *__restrict__ chunk, int64_t n, int64_t row0,
                                     double *P, double *E, double *OM, double *M0, double *S,
                                     float4 *mx_a, float4 *mx_b, float *mx_s2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double p = chunk[i * 5 + 0], e = chunk[i * 5 + 1], om = chunk[i * 5 + 2];
        const double m0 = chunk[i * 5 + 3], s = chunk[i * 5 + 4];
        const int64_t r = row0 + i;
        P[r] = p; E[r] = e; OM[r] = om; M0[r] = m0; S[r] = s;
        const double ip = 1.0 / p;
        const float ip_hi = (float)ip;
        const float ip_lo = (float)(ip - (double)ip_hi);
        double mc = m0 * INV_TWO_PI_D;
        mc -= floor(mc);                       // [0, 1)
        const float mc_hi = (float)mc;
        const float mc_lo = (float)(mc - (double)mc_hi);
        double sw, cw;
        sincos(om, &sw, &cw);
        // log g, g = P^(-2/3) / (1 - e^2): the per-sample factor of the
        // FixedCompanionMass variance sigma_K0^2 P0^(2/3) g
        const double lg = -2.0 / 3.0 * log(p) - log((1.0 - e) * (1.0 + e));
        mx_a[r] = make_float4(ip_hi, ip_lo, mc_hi, mc_lo);
        mx_b[r] = make_float4((float)e, (float)cw, (float)sw, (float)lg);
        mx_s2[r] = (float)(s * s);
    }
}

// ------------------------------------------------------------------ launchers
// Persistent launch: as many CTAs as can be resident on the device (never more
// than there are work items); each CTA loops over the shared work counter.
template <typename K>
static cudaError_t launch_persistent(K kern, const LnlArgs &a, int block, cudaStream_t st) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
    }
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, block, 0);
    if (e != cudaSuccess) return e;
    if (occ < 1) occ = 1;
    int grid = sms * occ;
    if (grid > a.n_items) grid = a.n_items;
    if (grid < 1) return cudaSuccess;
    kern<<<grid, block, 0, st>>>(a);
    return cudaGetLastError();
}

template <int L>
static cudaError_t launch_fp64_L(bool jit, const LnlArgs &a, int block, cudaStream_t st) {
    if (jit) return launch_persistent(lnl_fp64_kernel<L, true>, a, block, st);
    return launch_persistent(lnl_fp64_kernel<L, false>, a, block, st);
}

template <int L>
static cudaError_t launch_mixed_L(bool jit, bool acc, const LnlArgs &a, int block,
                                  cudaStream_t st) {
    if (jit) {
        if (acc) return launch_persistent(lnl_mixed_kernel<L, true, true>, a, block, st);
        return launch_persistent(lnl_mixed_kernel<L, true, false>, a, block, st);
    }
    if (acc) return launch_persistent(lnl_mixed_kernel<L, false, true>, a, block, st);
    return launch_persistent(lnl_mixed_kernel<L, false, false>, a, block, st);
}

cudaError_t launch_lnl(int precision, int L, bool jit, const LnlArgs &a, int block,
                       cudaStream_t st) {
    if (precision == JOKER_FP64) {
        switch (L) {
            case 1: return launch_fp64_L<1>(jit, a, block, st);
            case 2: return launch_fp64_L<2>(jit, a, block, st);
            case 3: return launch_fp64_L<3>(jit, a, block, st);
            case 4: return launch_fp64_L<4>(jit, a, block, st);
            case 5: return launch_fp64_L<5>(jit, a, block, st);
            case 6: return launch_fp64_L<6>(jit, a, block, st);
        }
    } else {
        const bool acc = precision == JOKER_MIXED_ACCURATE;
        switch (L) {
            case 1: return launch_mixed_L<1>(jit, acc, a, block, st);
            case 2: return launch_mixed_L<2>(jit, acc, a, block, st);
            case 3: return launch_mixed_L<3>(jit, acc, a, block, st);
            case 4: return launch_mixed_L<4>(jit, acc, a, block, st);
            case 5: return launch_mixed_L<5>(jit, acc, a, block, st);
            case 6: return launch_mixed_L<6>(jit, acc, a, block, st);
        }
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_prepare(const double *chunk, int64_t n, int64_t row0, double *P, double *E,
                           double *OM, double *M0, double *S, float4 *mx_a, float4 *mx_b,
                           float *mx_s2, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    prepare_cache_kernel<<<(int)blocks, 256, 0, st>>>(chunk, n, row0, P, E, OM, M0, S, mx_a, mx_b,
                                                      mx_s2);
    return cudaGetLastError();
}

}  // namespace joker
