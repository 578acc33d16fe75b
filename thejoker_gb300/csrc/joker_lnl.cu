// Marginal-likelihood kernels of libjoker_gb300 (sm_103a).
//
// For one star and one prior sample (P, e, omega, M0, s) the kernels evaluate
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
// columns (row 1 is the constant v0 term).  Without jitter everything that
// does not depend on the sample -- the trend block C of G, its inverse, the
// trend-only chi2_0 -- is folded per star on the host, so per sample only the
// Schur complement of the K column remains:
//   s = A00 + 1/Lambda0 - g^T C^-1 g,   u = b0 - g^T C^-1 c,
//   t = u - mu0 (s - 1/Lambda0),
//   chi2 = chi2_0 - 2 mu0 u + mu0^2 (s - 1/Lambda0) - t^2 / s,
//   log det G = log det C + log s.
// With the jitter applied the weights change per sample and the full L x L
// system is factorised per sample (LDL^T, K last).
//
// One thread owns one sample and walks the star's epochs, which the CTA
// stages in shared memory; CTAs pull (star, sample-range) work items from a
// global counter (a persistent launch sized to the SM count).
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
        if (it >= item_count(a)) break;
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
            const double P = a.P[row * a.stride];
            Acc64<L, JIT> acc;
            acc.init(st, P, a.e[row * a.stride], a.om[row * a.stride], a.M0[row * a.stride],
                     JIT ? a.s[row * a.stride] : 0.0);
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
                        acc.add(rec[0], rec[1], rec[2], rec + 3);
                    }
                }
            }
            double lnl = 0.0;
            if (active) {
                lnl = acc.finish(st, P);
                a.lnl[w.out_off + j] = lnl;
            }
            if (mk) warp_max_update(mk, active ? double_to_key(lnl) : 0ull);
        }
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
template <int L, bool JIT, int VAR>
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
        const float mu0f = st.mu0_f;
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
            // no jitter: A00 = sum w m^2, b0 = sum w m y', A0j = sum w m T_j
            float A00h = 0.f, A00l = 0.f, bh = 0.f, bl = 0.f;
            float Ah[MAXL], Al[MAXL];
#pragma unroll
            for (int k = 0; k < MAXL; ++k) { Ah[k] = 0.f; Al[k] = 0.f; }
            // jitter: sum w m^2, sum w r m, sum w m T_j, sum w T_j T_k,
            // sum w r T_j, sum w r^2, sum log2(1 + s^2 ivar)
            float GKKh = 0.f, GKKl = 0.f, qKh = 0.f, qKl = 0.f, rh = 0.f, rl = 0.f, lg2 = 0.f;
            float GKh[MAXL], GKl[MAXL], GTh[MAXL][MAXL], GTl[MAXL][MAXL], qTh[MAXL], qTl[MAXL];
            if (JIT) {
#pragma unroll
                for (int i = 0; i < MAXL; ++i) {
                    GKh[i] = GKl[i] = qTh[i] = qTl[i] = 0.f;
#pragma unroll
                    for (int k = 0; k < MAXL; ++k) GTh[i][k] = GTl[i][k] = 0.f;
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
                        kepler_sincos_f32<VAR == 1>(M, e, ome, a1, sE, cE);
                        const float den = __fmaf_rn(-e, cE, 1.0f);
                        float rd = fast_rcp(den);
                        rd = rd * __fmaf_rn(-den, rd, 2.0f);
                        const float m = __fmaf_rn(__fmaf_rn(Ac, cE, __fmaf_rn(Bc, sE, -Dc)), rd, Dc);
                        const float4 r1 = *reinterpret_cast<const float4 *>(rec + 4);
                        if (!JIT) {
                            float th, tl;                                 // w m, exact pair
                            two_prod(r0.z, m, th, tl);
                            tl = __fmaf_rn(r0.w, m, tl);
                            ff_acc(A00h, A00l, th, tl, m);
                            ff_acc(bh, bl, r1.x, r1.y, m);
                            if (L > 1) ff_add(Ah[1], Al[1], th, tl);      // T_1 = 1
#pragma unroll
                            for (int kk = 2; kk < L; ++kk)
                                ff_acc(Ah[kk], Al[kk], rec[4 + 2 * kk], rec[5 + 2 * kk], m);
                        } else {
                            const float iv = r0.z;
                            const float onep = __fmaf_rn(s2, iv, 1.0f);
                            float ro = fast_rcp(onep);
                            ro = ro * __fmaf_rn(-onep, ro, 2.0f);
                            const float wj = iv * ro;        // the weight, used consistently
                            lg2 += __log2f(onep);
                            // r = y' - mu0 m (float-float)
                            float rrh = r1.x, rrl = r1.y;
                            if (!mu0z) {
                                float ph, pl;
                                two_prod(-mu0f, m, ph, pl);
                                float s_, e_;
                                two_sum(rrh, ph, s_, e_);
                                rrl = __fadd_rn(__fadd_rn(rrl, e_), pl);
                                rrh = s_;
                            }
                            float wmh, wml;                                // w m, exact pair
                            two_prod(wj, m, wmh, wml);
                            float wrh, wrl;                                // w r
                            two_prod(wj, rrh, wrh, wrl);
                            wrl = __fmaf_rn(wj, rrl, wrl);
                            ff_acc(GKKh, GKKl, wmh, wml, m);
                            ff_acc(qKh, qKl, wrh, wrl, m);
                            if (L > 1) {                                   // T_1 = 1
                                ff_add(GKh[1], GKl[1], wmh, wml);
                                float t_, tl_;
                                two_sum(GTh[1][1], wj, t_, tl_);
                                GTh[1][1] = t_;
                                GTl[1][1] = __fadd_rn(GTl[1][1], tl_);
                                ff_add(qTh[1], qTl[1], wrh, wrl);
                            }
                            if (mu0z) {                                    // r^2 = y'^2, stored
                                const float p1 = __fmul_rn(wj, r1.z);
                                float pe1 = __fmaf_rn(wj, r1.z, -p1);
                                pe1 = __fmaf_rn(wj, r1.w, pe1);
                                ff_add(rh, rl, p1, pe1);
                            } else {
                                const float p1 = __fmul_rn(wrh, rrh);
                                float pe1 = __fmaf_rn(wrh, rrh, -p1);
                                pe1 = __fmaf_rn(wrh, rrl, __fmaf_rn(wrl, rrh, pe1));
                                ff_add(rh, rl, p1, pe1);
                            }
#pragma unroll
                            for (int ii = 2; ii < L; ++ii) {
                                const float Th = rec[6 + 2 * ii], Tl = rec[7 + 2 * ii];
                                {
                                    const float p2 = __fmul_rn(wmh, Th);
                                    float pe2 = __fmaf_rn(wmh, Th, -p2);
                                    pe2 = __fmaf_rn(wmh, Tl, __fmaf_rn(wml, Th, pe2));
                                    ff_add(GKh[ii], GKl[ii], p2, pe2);
                                }
                                {
                                    const float p2 = __fmul_rn(wrh, Th);
                                    float pe2 = __fmaf_rn(wrh, Th, -p2);
                                    pe2 = __fmaf_rn(wrh, Tl, __fmaf_rn(wrl, Th, pe2));
                                    ff_add(qTh[ii], qTl[ii], p2, pe2);
                                }
                                float wth, wtl;                            // w T_ii
                                two_prod(wj, Th, wth, wtl);
                                wtl = __fmaf_rn(wj, Tl, wtl);
                                ff_add(GTh[ii][1], GTl[ii][1], wth, wtl);
#pragma unroll
                                for (int kk = 2; kk <= ii; ++kk) {
                                    const float Tkh = rec[6 + 2 * kk], Tkl = rec[7 + 2 * kk];
                                    const float p2 = __fmul_rn(wth, Tkh);
                                    float pe2 = __fmaf_rn(wth, Tkh, -p2);
                                    pe2 = __fmaf_rn(wth, Tkl, __fmaf_rn(wtl, Tkh, pe2));
                                    ff_add(GTh[ii][kk], GTl[ii][kk], p2, pe2);
                                }
                            }
                        }
                    }
                }
            }
            double lnl = 0.0;
            float err = 0.0f;
            if (active) {
                // K prior variance: log Lambda0 from the per-sample log g
                float log_lam0f;
                if (st.k_scaled) log_lam0f = fminf((float)st.log_maxK2, (float)st.log_kscale + pb.w);
                else log_lam0f = (float)log(st.lam0);
                const float ilam0 = expf(-log_lam0f);
                float chi2f = 0.f, s_f = 1.f, amin_f = 0.f, Khat = 0.f, quadf = 0.f;
                if (VAR == 2) {
                    // FP64 tail (the literal FP64 form, kept for comparison)
                    const double lam0 = st.k_scaled ? (double)expf(log_lam0f) : st.lam0;
                    if (!JIT) {
                        double A0d[MAXL];
#pragma unroll
                        for (int kk = 0; kk < MAXL; ++kk) A0d[kk] = ff_to_double(Ah[kk], Al[kk]);
                        lnl = tail_schur_d<L, true>(st, ff_to_double(A00h, A00l), A0d,
                                                    ff_to_double(bh, bl), lam0, (double)log_lam0f);
                    } else {
                        double G[L][L], q[L];
                        G[0][0] = ff_to_double(GKKh, GKKl) + 1.0 / lam0;
                        q[0] = ff_to_double(qKh, qKl);
#pragma unroll
                        for (int ii = 1; ii < L; ++ii) {
                            G[ii][0] = G[0][ii] = ff_to_double(GKh[ii], GKl[ii]);
                            q[ii] = ff_to_double(qTh[ii], qTl[ii]);
#pragma unroll
                            for (int kk = 1; kk <= ii; ++kk)
                                G[ii][kk] = G[kk][ii] = ff_to_double(GTh[ii][kk], GTl[ii][kk]);
                            G[ii][ii] += 1.0 / st.lam[ii];
                        }
                        const double slw = st.sum_log_ivar - 0.6931471805599453 * (double)lg2;
                        lnl = tail_full_d<L, true>(G, q, ff_to_double(rh, rl),
                                                   st.log_norm_rest + (double)log_lam0f - slw);
                    }
                    err = 1e30f;   // this variant states no per-sample bound
                } else if (!JIT) {
                    // float-float Schur-complement tail
                    const ff A00 = ff_norm(A00h, A00l);
                    const ff b0 = ff_norm(bh, bl);
                    ff gv = ff_make(0.f, 0.f), gcC = ff_make(0.f, 0.f);
#pragma unroll
                    for (int jj = 1; jj < L; ++jj) {
                        const ff gj = ff_norm(Ah[jj], Al[jj]);
                        ff vj = ff_make(0.f, 0.f);
#pragma unroll
                        for (int kk = 1; kk < L; ++kk)
                            vj = ff_addf(vj, ff_mulf(ff_make(st.Cinv_hi[jj * MAXL + kk],
                                                             st.Cinv_lo[jj * MAXL + kk]),
                                                     ff_norm(Ah[kk], Al[kk])));
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
                        chi2 = ff_addf(chi2, ff_mul1(ff_subf(ff_mul1(amin, mu0f),
                                                             ff_mul1(u, 2.0f)), mu0f));
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
                        ff dk = ff_addf(ff_norm(GTh[k][k], GTl[k][k]), ff_make(st.ilam_hi[k], st.ilam_lo[k]));
#pragma unroll
                        for (int mm = 1; mm < k; ++mm) dk = ff_subf(dk, ff_mulf(ff_mulf(Lw[k][mm], Lw[k][mm]), Dd[mm]));
                        Dd[k] = dk;
#pragma unroll
                        for (int i = k + 1; i < L; ++i) {
                            ff v = ff_norm(GTh[i][k], GTl[i][k]);
#pragma unroll
                            for (int mm = 1; mm < k; ++mm) v = ff_subf(v, ff_mulf(ff_mulf(Lw[i][mm], Lw[k][mm]), Dd[mm]));
                            Lw[i][k] = ff_divf(v, dk);
                        }
                        ff v = ff_norm(GKh[k], GKl[k]);
#pragma unroll
                        for (int mm = 1; mm < k; ++mm) v = ff_subf(v, ff_mulf(ff_mulf(lK[mm], Lw[k][mm]), Dd[mm]));
                        lK[k] = ff_divf(v, dk);
                        logdet_G += ff_log(dk);
                    }
                    ff amin = ff_norm(GKKh, GKKl);
#pragma unroll
                    for (int k = 1; k < L; ++k) amin = ff_subf(amin, ff_mulf(ff_mulf(lK[k], lK[k]), Dd[k]));
                    const ff sK = ff_addf(amin, ff_make(ilam0, 0.f));
                    ff zK = ff_norm(qKh, qKl);
                    ff quad = ff_make(0.f, 0.f);
#pragma unroll
                    for (int k = 1; k < L; ++k) {
                        ff v = ff_norm(qTh[k], qTl[k]);
#pragma unroll
                        for (int mm = 1; mm < k; ++mm) v = ff_subf(v, ff_mulf(Lw[k][mm], z[mm]));
                        z[k] = v;
                        quad = ff_addf(quad, ff_divf(ff_mulf(v, v), Dd[k]));
                        zK = ff_subf(zK, ff_mulf(lK[k], v));
                    }
                    quad = ff_addf(quad, ff_divf(ff_mulf(zK, zK), sK));
                    logdet_G += ff_log(sK);
                    const ff chi2 = ff_subf(ff_norm(rh, rl), quad);
                    const double slw = st.sum_log_ivar - 0.6931471805599453 * (double)lg2;
                    lnl = -0.5 * (ff_to_d(chi2) + st.log_norm_rest + (double)log_lam0f +
                                  (double)logdet_G - slw);
                    chi2f = chi2.hi;
                    s_f = sK.hi;
                    amin_f = amin.hi;
                    Khat = zK.hi / sK.hi;
                    quadf = quad.hi;
                }
                if (VAR != 2) {
                    const float D = a.err_c0 * (1.0f + e) / (ome * ome);
                    const float Wsum = st.sum_ivar;
                    const float c2 = fmaxf(chi2f, 0.f);
                    const float dchi = 2.f * fabsf(Khat) * D * sqrtf(Wsum * c2) +
                                       Khat * Khat * D * D * Wsum;
                    const float ds = 2.f * D * sqrtf(Wsum * fmaxf(amin_f, 0.f)) + Wsum * D * D;
                    const float room = s_f - ds;
                    const float dlogs = (room > 1e-3f * s_f) ? ds / room : 1e30f;
                    err = 0.5f * (dchi + dlogs) + 2e-6f + 2e-7f * (float)N +
                          1e-12f * (fabsf(chi2f) + fabsf(quadf)) + (JIT ? 2e-7f * c2 : 0.f);
                    if (!(err == err)) err = 1e30f;      // NaN inputs: no bound
                }
                a.lnl[w.out_off + j] = lnl;
                if (a.err) a.err[w.out_off + j] = err;
            }
            if (mk) warp_max_update(mk, active ? double_to_key(lnl) : 0ull);
            if (bk) {
                warp_max_update(bk, active ? double_to_key(lnl + (double)err) : 0ull);
                warp_max_update(bk + 1, active ? double_to_key(lnl - (double)err) : 0ull);
            }
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
        // 1/P and M0/(2 pi) need their low words: FP64 (one division)
        const double ip = 1.0 / p;
        const float ip_hi = (float)ip;
        const float ip_lo = (float)(ip - (double)ip_hi);
        double mc = m0 * INV_TWO_PI_D;
        mc -= floor(mc);                       // [0, 1)
        const float mc_hi = (float)mc;
        const float mc_lo = (float)(mc - (double)mc_hi);
        // cos w, sin w and log g are stored as floats: FP32 is enough, with
        // the angle reduced to half-turns in FP64 first (sincospif is exact
        // in its argument reduction)
        double wc = om * 0.31830988618379067154;    // omega / pi
        wc -= 2.0 * floor(0.5 * wc);                // [0, 2)
        float sw, cw;
        sincospif((float)wc, &sw, &cw);
        // log g, g = P^(-2/3) / (1 - e^2): the per-sample factor of the
        // FixedCompanionMass variance sigma_K0^2 P0^(2/3) g
        const float lg = -0.6666667f * logf((float)p) - log1pf(-(float)(e * e));
        mx_a[r] = make_float4(ip_hi, ip_lo, mc_hi, mc_lo);
        mx_b[r] = make_float4((float)e, cw, sw, lg);
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
    if (!a.n_items_dev && grid > a.n_items) grid = a.n_items;
    if (grid < 1) return cudaSuccess;
    kern<<<grid, block, 0, st>>>(a);
    return cudaGetLastError();
}

template <int L>
static cudaError_t launch_fp64_L(bool jit, const LnlArgs &a, int block, cudaStream_t st) {
    if (jit) return launch_persistent(lnl_fp64_kernel<L, true>, a, block, st);
    return launch_persistent(lnl_fp64_kernel<L, false>, a, block, st);
}

template <int L, int VAR>
static cudaError_t launch_mixed_LV(bool jit, const LnlArgs &a, int block, cudaStream_t st) {
    if (jit) return launch_persistent(lnl_mixed_kernel<L, true, VAR>, a, block, st);
    return launch_persistent(lnl_mixed_kernel<L, false, VAR>, a, block, st);
}

template <int L>
static cudaError_t launch_mixed_L(bool jit, int var, const LnlArgs &a, int block,
                                  cudaStream_t st) {
    if (var == 1) return launch_mixed_LV<L, 1>(jit, a, block, st);
    if (var == 2) return launch_mixed_LV<L, 2>(jit, a, block, st);
    return launch_mixed_LV<L, 0>(jit, a, block, st);
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
        const int var = precision == JOKER_MIXED_ACCURATE ? 1
                      : precision == JOKER_MIXED_FP64_TAIL ? 2 : 0;
        switch (L) {
            case 1: return launch_mixed_L<1>(jit, var, a, block, st);
            case 2: return launch_mixed_L<2>(jit, var, a, block, st);
            case 3: return launch_mixed_L<3>(jit, var, a, block, st);
            case 4: return launch_mixed_L<4>(jit, var, a, block, st);
            case 5: return launch_mixed_L<5>(jit, var, a, block, st);
            case 6: return launch_mixed_L<6>(jit, var, a, block, st);
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
