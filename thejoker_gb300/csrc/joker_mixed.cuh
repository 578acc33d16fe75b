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
template <int L, bool JIT, int VAR, bool PACKED>
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
            float4 pa, pb;
            float s2;
            if (PACKED) {
                const int64_t q = row * a.stride;
                prepare_sample(__ldg(a.P + q), __ldg(a.e + q), __ldg(a.om + q), __ldg(a.M0 + q),
                               JIT ? __ldg(a.s + q) : 0.0, pa, pb, s2);
            } else {
                pa = __ldg(a.mx_a + row);
                pb = __ldg(a.mx_b + row);
                s2 = JIT ? __ldg(a.mx_s2 + row) : 0.0f;
            }
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

// Persistent launch: as many CTAs as can be resident on the device (never more
// than there are work items); each CTA loops over the shared work counter.
template <typename K>
inline cudaError_t launch_persistent(K kern, const LnlArgs &a, int block, cudaStream_t st) {
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

}  // namespace joker
