// Acceptance pass of libjoker_gb300: the reference's rejection step
//   uu = rng.uniform(size=len(lls))
//   good = np.where(np.exp(lls - lls.max()) > uu)[0][:max_posterior_samples]
// (thejoker/likelihood_helpers.py:107-109, multiproc_helpers.py:256-258),
// applied to many independent segments (stars / sample runs) at once.
//
// With mixed-precision ln L values and their per-sample error bounds the
// pass is exact with respect to FP64: a refine kernel first finds the FP64
// maximum among the samples whose interval [lnL - err, lnL + err] reaches the
// largest lower bound, and the mark kernel re-evaluates in FP64 every sample
// whose decision the interval leaves open.  Both touch a handful of samples.
//
// Three kernels, all bandwidth-bound scans over the ln L buffer:
//   mark  -- one warp per 1024 samples, lanes on consecutive samples (coalesced
//            loads); the test of 32 samples becomes one 32-bit word by ballot;
//            per-CTA accepted counts.
//   scan  -- exclusive scan of the per-CTA counts of each segment.
//   emit  -- per CTA, an in-block scan of word popcounts gives each accepted
//            sample its rank; indices are written in ascending order, the
//            first max_out of them only.
// The uniforms come either from a device array or from numpy's PCG64 stream,
// regenerated here from the generator state (joker_math.cuh), so the draws are
// bit-identical to rng.uniform() on the host.
#include <algorithm>

#include "joker_fp64.cuh"

namespace joker {

constexpr int ACC_THREADS = 256;                       // 8 warps
constexpr int64_t ACC_BLOCK = ACC_THREADS * 32;        // samples per CTA


__device__ __forceinline__ int find_seg(const AcceptArgs &a, int64_t b) {
    if (a.fixed_blocks > 0) return (int)(b / a.fixed_blocks);
    const int64_t *blk_base = a.blk_base;
    int lo = 0, hi = a.n_segs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (blk_base[mid] <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Number of 8192-sample blocks of this pass: the grid, or a device-side count
// when the pass runs inside a captured graph with a fixed grid.
__device__ __forceinline__ int64_t n_blocks(const AcceptArgs &a) {
    return a.total_blocks_dev ? *((volatile const int64_t *)a.total_blocks_dev) : (int64_t)gridDim.x;
}

__device__ __forceinline__ int64_t seg_base(const AcceptArgs &a, int si) {
    return a.fixed_blocks > 0 ? (int64_t)si * a.fixed_blocks : a.blk_base[si];
}

// exp(d) > u, evaluated as numpy does in FP64 but with an FP32 pre-test that
// settles all but the samples within 1e-4 of the boundary.
__device__ __forceinline__ bool accept_test(double d, double u) {
    if (!(d > -40.0)) {
        // exp(d) <= 4.3e-18 < 2^-53 <= any nonzero u; only u == 0 can pass
        return (u == 0.0) && (exp(d) > 0.0);
    }
    const float lf = __logf((float)u);
    const float df = (float)d;
    if (u > 0.0) {
        if (df > lf + 1e-4f) return true;
        if (df < lf - 1e-4f) return false;
    }
    return exp(d) > u;
}

// Decision for a sample known only to lie in [lnl - err, lnl + err]:
// 1 = keep, 0 = reject, -1 = undecided (needs the FP64 value).  The FP32
// log of u is trusted to 1e-4.
__device__ __forceinline__ int interval_test(double lnl, float err, double mx, double u) {
    if (!(err < 1e29f) || !(lnl == lnl)) return -1;
    const double dlo = lnl - (double)err - mx, dhi = lnl + (double)err - mx;
    if (u == 0.0) {
        if (dhi < -746.0) return 0;
        if (dlo > -744.0) return 1;
        return -1;
    }
    const float lf = __logf((float)u);
    if (dhi < -40.0 || (float)dhi < lf - 1e-4f) return 0;
    if ((float)dlo > lf + 1e-4f) return 1;
    return -1;
}

// ---- FP32 / integer fast paths -------------------------------------------
// GB300 runs FP64 (and FP64 conversions) at 1/64 of the FP32 rate, so the
// per-sample scans decide nearly every sample from float approximations built
// with integer operations, with margins that cover their error, and fall back
// to the FP64 tests above only near a decision boundary.

// float of a double by truncating its mantissa (relative error < 2^-23);
// false when the value is zero, subnormal in float, too large, inf or NaN.
__device__ __forceinline__ bool dbl_to_float_trunc(double x, float &f) {
    const long long b = __double_as_longlong(x);
    const int hi = (int)(b >> 32);
    const int ex = (hi >> 20) & 0x7ff;              // biased double exponent
    if (ex < 1023 - 126 || ex > 1023 + 127) return false;
    const unsigned mant = (unsigned)(b >> 29) & 0x7fffffu;
    f = __int_as_float((hi & (int)0x80000000) | ((ex - 1023 + 127) << 23) | (int)mant);
    return true;
}

// +infinity as a sample's bound: the ln L kernel found it out of reach, its
// ln L (upper bound) more than 746 nats below a lower bound of the maximum:
// exp(lnL - max) underflows to 0, so no uniform keeps it, and it is not the
// maximum.  (A tail without a bound writes 1e30, never +infinity.)
__device__ __forceinline__ bool out_of_reach(float er) {
    return __float_as_int(er) == 0x7f800000;
}

// Decision of exp(v + [-er, er] - mx) > u from float approximations:
// 1 keep, 0 reject, 2 undecided here (use the FP64 test).  uf = float u
// (> 0, truncated), vf, mxf = float approximations of v, mx.
__device__ __forceinline__ int fast_decide(float vf, float er, float mxf, float uf) {
    const float lu = __logf(uf);                     // |error| < 4e-7 + |log(1 + 2^-23)|
    const float tol = 1e-4f + 5e-7f * (fabsf(vf) + fabsf(mxf) + er);
    const float d = vf - mxf;
    if (d + er + tol < lu) return 0;
    if (d - er - tol > lu) return 1;
    return 2;
}

// Append a flagged sample to the compacted list (one atomic per warp);
// returns false for the samples that did not fit.
__device__ __forceinline__ bool flag_append(const AcceptArgs &a, int which, bool flag,
                                            int si, int64_t i) {
    const unsigned bal = __ballot_sync(0xffffffffu, flag);
    if (!bal) return true;
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == __ffs(bal) - 1) base = atomicAdd(a.flag_count + which, (unsigned long long)__popc(bal));
    base = __shfl_sync(0xffffffffu, base, __ffs(bal) - 1);
    if (!flag) return true;
    const int64_t pos = (int64_t)base + __popc(bal & ((1u << lane) - 1u));
    if (pos >= a.flag_cap) return false;
    a.flag_list[pos] = ((int64_t)si << 40) | i;
    return true;
}

// Candidates for each segment's FP64 maximum: the samples whose upper bound
// reaches the largest lower bound (the true maximum lies among them), plus
// samples without a usable bound.  Lean scan; marks bits in amb_words.
__global__ void __launch_bounds__(ACC_THREADS) accept_candidates_kernel(AcceptArgs a) {
    const int64_t nbk = n_blocks(a);
    for (int64_t gblk = blockIdx.x; gblk < nbk; gblk += gridDim.x) {
    const int si = find_seg(a, gblk);
    const joker_accept_seg sg = a.segs[si];
    const int64_t blk = gblk - seg_base(a, si);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t wbase = blk * ACC_BLOCK + (int64_t)warp * 1024;
    const double lb = key_to_double(a.bound_key[2 * sg.max_slot + 1]);
    float lbf;
    const bool fast = dbl_to_float_trunc(lb, lbf);
    uint32_t my_word = 0;
    for (int k = 0; k < 32; ++k) {
        const int64_t i = wbase + (int64_t)k * 32 + lane;
        bool cand = false;
        if (i < sg.n) {
            const double v = a.lnl[sg.lnl_off + i];
            const float er = a.err[sg.lnl_off + i];
            float vf;
            if (out_of_reach(er)) {
                cand = false;
            } else if (fast && er < 1e29f && dbl_to_float_trunc(v, vf) &&
                vf + er + (1e-6f + 5e-7f * (fabsf(vf) + fabsf(lbf) + er)) < lbf) {
                cand = false;                        // certainly below the largest lower bound
            } else {
                cand = (v + (double)er >= lb) || !(er < 1e29f) || !(v == v);
            }
        }
        const bool fit = flag_append(a, 0, cand, si, i);
        const uint32_t bal = __ballot_sync(0xffffffffu, !fit);
        if (lane == k) my_word = bal;
    }
    a.amb_words[gblk * ACC_THREADS + threadIdx.x] = my_word;
    }
}

// The maximum's refinement: a candidate whose interval -- tightened by the
// float-float tier, or as scanned -- no longer reaches the star's largest
// lower bound (raised by that tier) cannot be the maximum.
__device__ __forceinline__ bool below_lower_bound(const AcceptArgs &a, const joker_accept_seg &sg,
                                                  int64_t i) {
    const double v = a.lnl[sg.lnl_off + i];
    const float er = a.err[sg.lnl_off + i];
    if (!(er < 1e29f) || !(v == v)) return false;
    return v + (double)er < key_to_double(a.bound_key[2 * sg.max_slot + 1]);
}

// FP64 work on the samples flagged in amb_words (the lists' overflow).  One
// thread covers
// WORDS_PER_THREAD consecutive words (all inside one 256-word CTA block);
// almost all words are zero.  MODE 0 raises the FP64 maximum; MODE 1 decides
// the undecided samples against it and their own uniforms; MODE 2 writes the
// FP64 value back.
constexpr int WORDS_PER_THREAD = 16;

template <int MODE>
__device__ __noinline__ void fp64_words_phase(const AcceptArgs &a, int64_t n_words) {
    if (a.total_blocks_dev) n_words = n_blocks(a) * ACC_THREADS;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
         t * WORDS_PER_THREAD < n_words; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t w0 = t * WORDS_PER_THREAD;
    uint32_t wv[WORDS_PER_THREAD];
    const uint4 *p = reinterpret_cast<const uint4 *>(a.amb_words + w0);
    bool any = false;
#pragma unroll
    for (int q = 0; q < WORDS_PER_THREAD / 4; ++q) {
        const uint4 v = p[q];
        wv[4 * q] = v.x; wv[4 * q + 1] = v.y; wv[4 * q + 2] = v.z; wv[4 * q + 3] = v.w;
        any |= (v.x | v.y | v.z | v.w) != 0u;
    }
    if (!any) continue;
    if (MODE != 1) {
        // consumed: cleared, so that a later pass can flag into zero words
        uint4 *pw = reinterpret_cast<uint4 *>(a.amb_words + w0);
#pragma unroll
        for (int q = 0; q < WORDS_PER_THREAD / 4; ++q) pw[q] = make_uint4(0u, 0u, 0u, 0u);
    }
    const int64_t gblk = w0 / ACC_THREADS;
    const int si = find_seg(a, gblk);
    const joker_accept_seg sg = a.segs[si];
    const int64_t blk = gblk - seg_base(a, si);
    const double mx = MODE == 1 ? key_to_double(a.exact_key[sg.max_slot]) : 0.0;
    for (int q = 0; q < WORDS_PER_THREAD; ++q) {
        uint32_t bits = wv[q];
        if (!bits) continue;
        const int64_t wi = w0 + q;                                 // global word
        const int64_t first = blk * ACC_BLOCK + (wi - gblk * ACC_THREADS) * 32;
        uint32_t add = 0;
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1;
            const int64_t i = first + b;
            if (i >= sg.n) continue;
            if (MODE == 0 && below_lower_bound(a, sg, i)) continue;
            const bool exact = a.err[sg.lnl_off + i] == 0.0f;
            const int64_t r = (sg.row0 + i) * a.stride;
            const double v = exact ? a.lnl[sg.lnl_off + i]
                                   : fp64_lnl_sample(a.L, a.jit, a.stars[sg.star], a.ep64,
                                                     a.P[r], a.E[r], a.OM[r], a.M0[r], a.S[r]);
            if (a.n_refined && !exact) atomicAdd(a.n_refined, 1ull);
            if (MODE == 0) {
                atomicMax(a.exact_key + sg.max_slot, double_to_key(v));
                if (a.write_max) {
                    const_cast<double *>(a.lnl)[sg.lnl_off + i] = v;
                    const_cast<float *>(a.err)[sg.lnl_off + i] = 0.0f;
                }
            } else if (MODE == 2) {
                const_cast<double *>(a.lnl)[sg.lnl_off + i] = v;
                const_cast<float *>(a.err)[sg.lnl_off + i] = 0.0f;
            } else {
                double u;
                if (a.u_source == JOKER_U_PCG64) {
                    const u128 s0 = ((u128)sg.pcg_state_hi << 64) | (u128)sg.pcg_state_lo;
                    const u128 inc = ((u128)sg.pcg_inc_hi << 64) | (u128)sg.pcg_inc_lo;
                    u = pcg_uniform(pcg_output(pcg_jump(s0, inc, (uint64_t)i + 1)));
                } else {
                    u = a.u[sg.u_off + i];
                }
                const_cast<double *>(a.lnl)[sg.lnl_off + i] = v;
                const_cast<float *>(a.err)[sg.lnl_off + i] = 0.0f;
                if (accept_test(v - mx, u)) add |= 1u << b;
            }
        }
        if (MODE == 1 && add) {
            atomicOr(a.words + wi, add);
            atomicAdd((unsigned long long *)(a.blk_count + gblk), (unsigned long long)__popc(add));
        }
    }
    }
}

// FP64 re-evaluation of the listed samples, one warp per sample (lanes over
// epochs), then (scan_words) of the samples flagged in amb_words past the
// list's capacity.  MODE 0 raises the FP64 maximum; MODE 1 decides the
// undecided samples against it and their own uniforms; MODE 2 (the band
// refinement) only writes the FP64 value back.  n_words: words of amb_words
// (read from the device count when the pass has one).
template <int MODE>
__global__ void __launch_bounds__(256, 2) accept_fp64_list_kernel(AcceptArgs a, int64_t n_words,
                                                                    int scan_words) {
    const int lane = threadIdx.x & 31;
    const int64_t n = min((int64_t)a.flag_count[MODE == 1 ? 1 : 0], a.flag_cap);   // MODE 2 uses list 0
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t e = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); e < n;
         e += nw) {
        const int64_t ent = a.flag_list[e];
        const int si = (int)(ent >> 40);
        const int64_t i = ent & (((int64_t)1 << 40) - 1);
        const joker_accept_seg sg = a.segs[si];
        if (MODE == 0 && below_lower_bound(a, sg, i)) continue;     // uniform in the warp
        // a value an earlier refinement made exact (bound 0) is not evaluated again
        const bool exact = a.err[sg.lnl_off + i] == 0.0f;
        const int64_t r = (sg.row0 + i) * a.stride;
        const double v = exact ? a.lnl[sg.lnl_off + i]
                               : fp64_lnl_warp(a.L, a.jit, a.stars[sg.star], a.ep64, a.P[r],
                                               a.E[r], a.OM[r], a.M0[r], a.S[r]);
        if (lane != 0) continue;
        if (a.n_refined && !exact) atomicAdd(a.n_refined, 1ull);
        if (MODE == 0) {
            atomicMax(a.exact_key + sg.max_slot, double_to_key(v));
            if (a.write_max) {
                const_cast<double *>(a.lnl)[sg.lnl_off + i] = v;
                const_cast<float *>(a.err)[sg.lnl_off + i] = 0.0f;
            }
        } else if (MODE == 2) {
            const_cast<double *>(a.lnl)[sg.lnl_off + i] = v;
            const_cast<float *>(a.err)[sg.lnl_off + i] = 0.0f;
        } else {
            const double mx = key_to_double(a.exact_key[sg.max_slot]);
            double u;
            if (a.u_source == JOKER_U_PCG64) {
                const u128 s0 = ((u128)sg.pcg_state_hi << 64) | (u128)sg.pcg_state_lo;
                const u128 inc = ((u128)sg.pcg_inc_hi << 64) | (u128)sg.pcg_inc_lo;
                u = pcg_uniform(pcg_output(pcg_jump(s0, inc, (uint64_t)i + 1)));
            } else {
                u = a.u[sg.u_off + i];
            }
            // the FP64 value replaces the mixed one (exact, so its bound is 0)
            const_cast<double *>(a.lnl)[sg.lnl_off + i] = v;
            const_cast<float *>(a.err)[sg.lnl_off + i] = 0.0f;
            if (accept_test(v - mx, u)) {
                const int64_t gblk = seg_base(a, si) + i / ACC_BLOCK;
                atomicOr(a.words + gblk * ACC_THREADS + (i % ACC_BLOCK) / 32, 1u << (i & 31));
                atomicAdd((unsigned long long *)(a.blk_count + gblk), 1ull);
            }
        }
    }
    if (scan_words) fp64_words_phase<MODE>(a, n_words);
}

// The band refinement's scan: flags every sample whose mixed interval reaches
// within `band` of its slot's FP64 maximum (lnL + err >= max - band) and whose
// bound exceeds `tol`, and every sample without a usable bound or value.  The
// float pre-test settles the samples far below the band without FP64 work.
__global__ void __launch_bounds__(ACC_THREADS) band_flag_kernel(AcceptArgs a, double band,
                                                                float tol) {
    const int64_t nbk = n_blocks(a);
    for (int64_t gblk = blockIdx.x; gblk < nbk; gblk += gridDim.x) {
    const int si = find_seg(a, gblk);
    const joker_accept_seg sg = a.segs[si];
    const int64_t blk = gblk - seg_base(a, si);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t wbase = blk * ACC_BLOCK + (int64_t)warp * 1024;
    const double thr = key_to_double(a.exact_key[sg.max_slot]) - band;
    float thrf;
    const bool fast = dbl_to_float_trunc(thr, thrf);
    uint32_t my_word = 0;
    for (int k = 0; k < 32; ++k) {
        const int64_t i = wbase + (int64_t)k * 32 + lane;
        bool flag = false;
        if (i < sg.n) {
            const double v = a.lnl[sg.lnl_off + i];
            const float er = a.err[sg.lnl_off + i];
            float vf;
            if (out_of_reach(er)) {
                flag = band >= 746.0;                // more than 746 below the maximum
            } else if (!(er < 1e29f) || !(v == v)) {
                flag = true;                         // no bound, or no value
            } else if (er <= tol) {
                flag = false;                        // already within the tolerance
            } else if (fast && dbl_to_float_trunc(v, vf) &&
                       vf + er + (1e-6f + 5e-7f * (fabsf(vf) + fabsf(thrf) + er)) < thrf) {
                flag = false;                        // certainly below the band
            } else {
                flag = v + (double)er >= thr;
            }
        }
        const bool fit = flag_append(a, 0, flag, si, i);
        const uint32_t bal = __ballot_sync(0xffffffffu, !fit);
        if (lane == k) my_word = bal;
    }
    a.amb_words[gblk * ACC_THREADS + threadIdx.x] = my_word;
    }
}

__global__ void __launch_bounds__(ACC_THREADS) accept_mark_kernel(AcceptArgs a) {
    __shared__ int s_cnt[ACC_THREADS / 32];
    const int64_t nbk = n_blocks(a);
    for (int64_t gblk = blockIdx.x; gblk < nbk; gblk += gridDim.x) {
    const int si = find_seg(a, gblk);
    const joker_accept_seg sg = a.segs[si];
    const int64_t blk = gblk - seg_base(a, si);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t wbase = blk * ACC_BLOCK + (int64_t)warp * 1024;  // first sample of this warp
    const bool refine = a.err != nullptr;
    const double mx = refine ? key_to_double(a.exact_key[sg.max_slot])
                             : key_to_double(a.max_key[sg.max_slot]);
    const double *lnl = a.lnl + sg.lnl_off;

    // four independent PCG64 chains per lane (k = 4 kk + c, c = 0..3), each
    // stepping 128 positions: draw at position p is output(state after p + 1 steps)
    u128 stc[4] = {0, 0, 0, 0}, inc = 0, A128 = 1, C128 = 0;
    if (a.u_source == JOKER_U_PCG64) {
        const u128 s0 = ((u128)sg.pcg_state_hi << 64) | (u128)sg.pcg_state_lo;
        inc = ((u128)sg.pcg_inc_hi << 64) | (u128)sg.pcg_inc_lo;
        const u128 sw = pcg_jump(s0, inc, (uint64_t)(wbase + 1));     // uniform over the warp
        stc[0] = u128_of(g_pcg.lane_a[lane]) * sw + u128_of(g_pcg.lane_s[lane]) * inc;
        const u128 A32 = u128_of(g_pcg.lane_a[32]), C32 = u128_of(g_pcg.lane_s[32]) * inc;
#pragma unroll
        for (int c = 1; c < 4; ++c) stc[c] = A32 * stc[c - 1] + C32;
        A128 = u128_of(g_pcg.dbl_a[7]);
        C128 = u128_of(g_pcg.dbl_s[7]) * inc;
    }
    float mxf;
    const bool fast = dbl_to_float_trunc(mx, mxf);
    uint32_t my_word = 0, my_amb = 0;
    int my_count = 0;
    for (int kk = 0; kk < 8; ++kk) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const int k = 4 * kk + c;
        const u128 st = stc[c];
        const int64_t i = wbase + (int64_t)k * 32 + lane;
        bool keep = false, amb = false;
        if (i < sg.n) {
            // the uniform: its 53-bit integer (PCG64) or the array's double
            uint64_t m = 0;
            double ua = 0.0;
            float uf = 0.0f;
            bool uf_ok;
            if (a.u_source == JOKER_U_PCG64) {
                m = pcg_output(st) >> 11;
                uf_ok = m != 0;
                if (uf_ok) uf = u53_to_float(m);
            } else {
                ua = a.u[sg.u_off + i];
                uf_ok = dbl_to_float_trunc(ua, uf);
            }
            const double v = lnl[i];
            const float er = refine ? a.err[sg.lnl_off + i] : 0.0f;
            float vf;
            int dec = 2;
            if (refine && out_of_reach(er))
                dec = 0;
            else if (fast && uf_ok && er < 1e29f && dbl_to_float_trunc(v, vf))
                dec = fast_decide(vf, er, mxf, uf);
            if (dec == 2) {
                const double u = a.u_source == JOKER_U_PCG64 ? (double)m * 0x1.0p-53 : ua;
                if (!refine) {
                    dec = accept_test(v - mx, u) ? 1 : 0;
                } else {
                    dec = interval_test(v, er, mx, u);
                }
            }
            keep = dec == 1;
            amb = dec < 0;
        }
        if (a.u_source == JOKER_U_PCG64) stc[c] = A128 * stc[c] + C128;
        const uint32_t bal = __ballot_sync(0xffffffffu, keep);
        const bool fit = !refine || flag_append(a, 1, amb, si, i);
        const uint32_t abal = __ballot_sync(0xffffffffu, !fit);
        if (lane == k) {
            my_word = bal;
            my_amb = abal;
        }
        my_count += __popc(bal);
    }
    }
    // word index within the CTA: warp * 32 + lane
    a.words[gblk * ACC_THREADS + threadIdx.x] = my_word;
    if (refine) a.amb_words[gblk * ACC_THREADS + threadIdx.x] = my_amb;
    if (lane == 0) s_cnt[warp] = my_count;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t c = 0;
        for (int w = 0; w < ACC_THREADS / 32; ++w) c += s_cnt[w];
        a.blk_count[gblk] = c;
    }
    __syncthreads();
    }
}

// ---- second stage of the fused pass -----------------------------------------
// The ln L kernel has left one candidate bit per sample (cand_words); every
// sample without it is rejected.  These scans read the bits (1/96 of the
// bytes of ln L and its bound) and touch ln L only where a bit is set.

__device__ __forceinline__ uint32_t cand_word(const AcceptArgs &a, int si, int64_t n,
                                              int64_t first) {
    if (first >= n) return 0u;
    uint32_t w = a.cand_words[(int64_t)si * a.cand_ld + (first >> 5)];
    if (n - first < 32) w &= (1u << (n - first)) - 1u;
    return w;
}

// Both scans take one 8192-sample CTA block per warp (grid-stride): each lane
// loads 8 of the block's 256 words of candidate bits (two 16-byte loads, all
// independent), and only the nonzero words are visited, each by the whole
// warp (lane b on the word's sample b).  The arrays they fill (amb_words,
// words) and the per-CTA counts are zeroed before; a block without candidate
// bits costs its loads.
struct FusedBlock {
    int si;
    joker_accept_seg sg;
    int64_t gblk, first;      // CTA block; its first sample in the segment
    uint32_t wv[8];           // words 8 lane .. 8 lane + 7 of the block
};

__device__ __forceinline__ void fused_block(const AcceptArgs &a, int64_t gblk, FusedBlock &b) {
    const int lane = threadIdx.x & 31;
    b.gblk = gblk;
    b.si = find_seg(a, gblk);
    b.sg = a.segs[b.si];
    b.first = (gblk - seg_base(a, b.si)) * ACC_BLOCK;
    const int64_t nw = (b.sg.n + 31) >> 5;                  // words of the segment
    const int64_t w0 = (b.first >> 5) + 8 * lane;
    const uint32_t *row = a.cand_words + (int64_t)b.si * a.cand_ld;
    if (w0 + 8 <= nw) {
        const uint4 p = *reinterpret_cast<const uint4 *>(row + w0);
        const uint4 q = *reinterpret_cast<const uint4 *>(row + w0 + 4);
        b.wv[0] = p.x; b.wv[1] = p.y; b.wv[2] = p.z; b.wv[3] = p.w;
        b.wv[4] = q.x; b.wv[5] = q.y; b.wv[6] = q.z; b.wv[7] = q.w;
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) b.wv[j] = w0 + j < nw ? row[w0 + j] : 0u;
    }
    // the segment's last word: bits past its last sample
    const int64_t tail = b.sg.n & 31;
    if (tail) {
#pragma unroll
        for (int j = 0; j < 8; ++j)
            if (w0 + j == nw - 1) b.wv[j] &= (1u << tail) - 1u;
    }
}

// Visit every nonzero word of the block: fn(word index in the block, bits),
// called by all lanes (warp-uniform).
template <class F>
__device__ __forceinline__ void for_nonzero_words(const FusedBlock &b, F fn) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        unsigned owners = __ballot_sync(0xffffffffu, b.wv[j] != 0u);
        while (owners) {
            const int l = __ffs(owners) - 1;
            owners &= owners - 1;
            fn(8 * l + j, __shfl_sync(0xffffffffu, b.wv[j], l));
        }
    }
}

// Candidates for each segment's FP64 maximum: the candidate samples whose
// upper bound reaches the largest lower bound, plus those without a usable
// bound (as accept_candidates_kernel, over the bits only); flag list 0,
// past its capacity bits in amb_words.
__global__ void __launch_bounds__(ACC_THREADS) fused_max_cands_kernel(AcceptArgs a, int64_t nbk) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (ACC_THREADS / 32);
    for (int64_t gblk = blockIdx.x * (int64_t)(ACC_THREADS / 32) + (threadIdx.x >> 5);
         gblk < nbk; gblk += nwarps) {
        FusedBlock b;
        fused_block(a, gblk, b);
        const double lb = key_to_double(a.bound_key[2 * b.sg.max_slot + 1]);
        for_nonzero_words(b, [&](int w, uint32_t bits) {
            const int64_t i = b.first + 32 * w + lane;
            bool cand = false;
            if ((bits >> lane) & 1u) {
                const double v = a.lnl[b.sg.lnl_off + i];
                const float er = a.err[b.sg.lnl_off + i];
                cand = (v + (double)er >= lb) || !(er < 1e29f) || !(v == v);
            }
            const uint32_t over = __ballot_sync(0xffffffffu, !flag_append(a, 0, cand, b.si, i));
            if (over && lane == 0) a.amb_words[gblk * ACC_THREADS + w] = over;
        });
    }
}

// The decisions: the mark pass over the candidate bits.  For each nonzero
// word its 32 lanes regenerate their uniforms -- the block's state by one
// jump, then a table step to the word and one to the lane -- and decide the
// candidates against the FP64 maximum as the mark pass does; kept bits go
// to words, undecided samples to flag list 1 (past its capacity to
// amb_words), the kept count to the block's counter.
__global__ void __launch_bounds__(ACC_THREADS) fused_decide_kernel(AcceptArgs a, int64_t nbk) {
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = (int64_t)gridDim.x * (ACC_THREADS / 32);
    for (int64_t gblk = blockIdx.x * (int64_t)(ACC_THREADS / 32) + (threadIdx.x >> 5);
         gblk < nbk; gblk += nwarps) {
        FusedBlock b;
        fused_block(a, gblk, b);
        bool any = false;
#pragma unroll
        for (int j = 0; j < 8; ++j) any |= b.wv[j] != 0u;
        if (!__any_sync(0xffffffffu, any)) continue;
        const double mx = key_to_double(a.exact_key[b.sg.max_slot]);
        float mxf;
        const bool fast = dbl_to_float_trunc(mx, mxf);
        const u128 inc = ((u128)b.sg.pcg_inc_hi << 64) | (u128)b.sg.pcg_inc_lo;
        const u128 sblk = pcg_jump(((u128)b.sg.pcg_state_hi << 64) | (u128)b.sg.pcg_state_lo, inc,
                                   (uint64_t)b.first);
        const unsigned long long *lt = g_pcg_thr.v[lane];
        const u128 a_lane = ((u128)lt[1] << 64) | (u128)lt[0];
        const u128 c_lane = (((u128)lt[3] << 64) | (u128)lt[2]) * inc;
        int count = 0;
        for_nonzero_words(b, [&](int w, uint32_t bits) {
            const int64_t i = b.first + 32 * w + lane;
            const unsigned long long *wt = g_pcg_w32.v[w];
            const u128 sw = (((u128)wt[1] << 64) | (u128)wt[0]) * sblk +
                            (((u128)wt[3] << 64) | (u128)wt[2]) * inc;
            bool keep = false, amb = false;
            if ((bits >> lane) & 1u) {
                const uint64_t m = pcg_output(a_lane * sw + c_lane) >> 11;
                const double v = a.lnl[b.sg.lnl_off + i];
                const float er = a.err[b.sg.lnl_off + i];
                float vf;
                int dec = 2;
                if (fast && m != 0 && er < 1e29f && dbl_to_float_trunc(v, vf))
                    dec = fast_decide(vf, er, mxf, u53_to_float(m));
                if (dec == 2) dec = interval_test(v, er, mx, (double)m * 0x1.0p-53);
                keep = dec == 1;
                amb = dec < 0;
            }
            const uint32_t bal = __ballot_sync(0xffffffffu, keep);
            const uint32_t over = __ballot_sync(0xffffffffu, !flag_append(a, 1, amb, b.si, i));
            if (lane == 0) {
                if (bal) a.words[gblk * ACC_THREADS + w] = bal;
                if (over) a.amb_words[gblk * ACC_THREADS + w] = over;
            }
            count += __popc(bal);
        });
        if (lane == 0 && count)
            atomicAdd((unsigned long long *)(a.blk_count + gblk), (unsigned long long)count);
    }
}

// One CTA per segment: exclusive scan of that segment's per-CTA counts,
// SCAN_PER consecutive counts per thread (SCAN_THREADS x SCAN_PER per round),
// warp shuffles for the block-wide part.
constexpr int SCAN_THREADS = 1024, SCAN_PER = 8;

__global__ void __launch_bounds__(SCAN_THREADS) accept_scan_kernel(AcceptArgs a) {
    const int si = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t b0 = seg_base(a, si), nb = seg_base(a, si + 1) - b0;
    __shared__ int64_t s_w[SCAN_THREADS / 32];
    int64_t carry = 0;
    for (int64_t base = 0; base < nb; base += (int64_t)SCAN_THREADS * SCAN_PER) {
        const int64_t e0 = base + (int64_t)threadIdx.x * SCAN_PER;
        int64_t v[SCAN_PER], sum = 0;
#pragma unroll
        for (int j = 0; j < SCAN_PER; ++j) {
            v[j] = e0 + j < nb ? a.blk_count[b0 + e0 + j] : 0;
            sum += v[j];
        }
        int64_t x = sum;                                   // inclusive scan in the warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) s_w[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int64_t t = s_w[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            s_w[lane] = t;
        }
        __syncthreads();
        int64_t run = carry + (warp ? s_w[warp - 1] : 0) + x - sum;
#pragma unroll
        for (int j = 0; j < SCAN_PER; ++j) {
            if (e0 + j < nb) a.blk_count[b0 + e0 + j] = run;
            run += v[j];
        }
        carry += s_w[SCAN_THREADS / 32 - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) a.count[si] = carry;
}

// Emit: each accepted sample's rank in its segment; the first max_out of them
// are written out.  FLAG (refined pass with ln L outputs, before the writing
// pass): every output sample whose bound exceeds JOKER_MIXED_LNL_TOL is put
// on flag list 0 for re-evaluation in FP64 (or, past the list's capacity,
// re-evaluated here), so that every ln L written out is within that of FP64.
template <bool FLAG>
__global__ void __launch_bounds__(ACC_THREADS) accept_emit_kernel(AcceptArgs a) {
    __shared__ int s_scan[ACC_THREADS];
    const int64_t nbk = n_blocks(a);
    for (int64_t gblk = blockIdx.x; gblk < nbk; gblk += gridDim.x) {
    const int si = find_seg(a, gblk);
    const joker_accept_seg sg = a.segs[si];
    const int64_t blk = gblk - seg_base(a, si);
    const int64_t boff = a.blk_count[gblk];
    if (boff >= sg.max_out) continue;
    // nothing kept in this block: the next block's offset (or the segment's
    // count) equals this one's
    const int64_t bnext = gblk + 1 < seg_base(a, si + 1) ? a.blk_count[gblk + 1] : a.count[si];
    if (bnext == boff) continue;
    const uint32_t word = a.words[gblk * ACC_THREADS + threadIdx.x];
    const int c = __popc(word);
    s_scan[threadIdx.x] = c;
    __syncthreads();
    for (int off = 1; off < ACC_THREADS; off <<= 1) {
        const int add = (threadIdx.x >= off) ? s_scan[threadIdx.x - off] : 0;
        __syncthreads();
        s_scan[threadIdx.x] += add;
        __syncthreads();
    }
    int64_t pos = boff + s_scan[threadIdx.x] - c;
    const int64_t first = blk * ACC_BLOCK + (int64_t)threadIdx.x * 32;
    uint32_t wm = word;
    while (wm && pos < sg.max_out) {
        const int b = __ffs(wm) - 1;
        wm &= wm - 1;
        const int64_t i = first + b;
        if (FLAG) {
            if (!(a.err[sg.lnl_off + i] <= (float)JOKER_MIXED_LNL_TOL)) {
                const unsigned long long q = atomicAdd(a.flag_count, 1ull);
                if ((int64_t)q < a.flag_cap) {
                    a.flag_list[q] = ((int64_t)si << 40) | i;
                } else {
                    const int64_t r = (sg.row0 + i) * a.stride;
                    const double v = fp64_lnl_sample(a.L, a.jit, a.stars[sg.star], a.ep64,
                                                     a.P[r], a.E[r], a.OM[r], a.M0[r], a.S[r]);
                    if (a.n_refined) atomicAdd(a.n_refined, 1ull);
                    const_cast<double *>(a.lnl)[sg.lnl_off + i] = v;
                    const_cast<float *>(a.err)[sg.lnl_off + i] = 0.0f;
                }
            }
        } else {
            a.out_idx[sg.out_off + pos] = sg.idx_base + i;
            if (a.out_lnl) a.out_lnl[sg.out_off + pos] = a.lnl[sg.lnl_off + i];
        }
        ++pos;
    }
    __syncthreads();
    }
}

int64_t accept_blocks(const joker_accept_seg *segs, int n_segs, int64_t *blk_base_host) {
    int64_t tot = 0;
    for (int s = 0; s < n_segs; ++s) {
        if (blk_base_host) blk_base_host[s] = tot;
        tot += (segs[s].n + ACC_BLOCK - 1) / ACC_BLOCK;
    }
    if (blk_base_host) blk_base_host[n_segs] = tot;
    return tot;
}

// Loads the module of the plain pass's kernels (mark, scan, emit) on the
// current device without launching them.  Under lazy module loading (the
// default since CUDA 12.2) a module is loaded, and its device memory taken, at
// the first use of one of its functions; joker_accept_noalloc's warm-up call
// uses this so that no later call loads anything.
cudaError_t accept_preload() {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, accept_mark_kernel);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, accept_scan_kernel);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, accept_emit_kernel<false>);
    return e;
}

static cudaError_t launch_fp64_words(int mode, const AcceptArgs &a, int64_t total_blocks,
                                     cudaStream_t st) {
    // the compacted list (one warp per sample), then the words of the samples
    // that did not fit in it (almost always none), in one launch
    const unsigned grid = 152 * 4;
    const int64_t n_words = total_blocks * ACC_THREADS;
    if (mode == 0) accept_fp64_list_kernel<0><<<grid, 256, 0, st>>>(a, n_words, 1);
    else if (mode == 1) accept_fp64_list_kernel<1><<<grid, 256, 0, st>>>(a, n_words, 1);
    else accept_fp64_list_kernel<2><<<grid, 256, 0, st>>>(a, n_words, 1);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_refine_band(const AcceptArgs &a, int64_t total_blocks, double band, float tol,
                               cudaStream_t st) {
    if (total_blocks <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(a.flag_count, 0, 2 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    band_flag_kernel<<<(unsigned)total_blocks, ACC_THREADS, 0, st>>>(a, band, tol);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return launch_fp64_words(2, a, total_blocks, st);
}

cudaError_t launch_tier2(const AcceptArgs &a, cudaStream_t st);

cudaError_t launch_refine_max(const AcceptArgs &a, int64_t total_blocks, cudaStream_t st) {
    if (total_blocks <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(a.flag_count, 0, 2 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    accept_candidates_kernel<<<(unsigned)total_blocks, ACC_THREADS, 0, st>>>(a);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // the float-float tier tightens the listed candidates and raises the
    // lower bounds; FP64 then takes only those still reaching them
    e = launch_tier2(a, st);
    if (e != cudaSuccess) return e;
    return launch_fp64_words(0, a, total_blocks, st);
}

static cudaError_t accept_finish(const AcceptArgs &a, int64_t total_blocks, cudaStream_t st);

cudaError_t launch_accept(const AcceptArgs &a, int64_t total_blocks, cudaStream_t st,
                          bool max_given) {
    if (a.err != nullptr && !max_given && total_blocks > 0) {
        cudaError_t e = launch_refine_max(a, total_blocks, st);
        if (e != cudaSuccess) return e;
    }
    if (total_blocks > 0) {
        cudaError_t e;
        if (a.err != nullptr &&
            (e = cudaMemsetAsync(a.flag_count + 1, 0, sizeof(unsigned long long), st)) != cudaSuccess)
            return e;
        accept_mark_kernel<<<(unsigned)total_blocks, ACC_THREADS, 0, st>>>(a);
        count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (a.err != nullptr) {
            e = launch_fp64_words(1, a, total_blocks, st);
            if (e != cudaSuccess) return e;
        }
    }
    return accept_finish(a, total_blocks, st);
}

// The fused pass's second stage, after the ln L kernel has written the
// candidate bits (a.cand_words) and the bound maxima; a.exact_key zeroed.
// The flag words of list 0's overflow are cleared by the FP64 pass that
// reads them, so list 1's overflow starts from zero words too.
cudaError_t launch_accept_fused(const AcceptArgs &a, int64_t total_blocks, cudaStream_t st) {
    if (total_blocks > 0) {
        const unsigned grid = (unsigned)std::min<int64_t>((total_blocks + 7) / 8, 152 * 8);
        const size_t wbytes = (size_t)total_blocks * ACC_THREADS * sizeof(uint32_t);
        cudaError_t e = cudaMemsetAsync(a.flag_count, 0, 2 * sizeof(unsigned long long), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(a.amb_words, 0, wbytes, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(a.words, 0, wbytes, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(a.blk_count, 0, 8 * (size_t)total_blocks, st);
        if (e != cudaSuccess) return e;
        fused_max_cands_kernel<<<grid, ACC_THREADS, 0, st>>>(a, total_blocks);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = launch_tier2(a, st)) != cudaSuccess) return e;
        if ((e = launch_fp64_words(0, a, total_blocks, st)) != cudaSuccess) return e;
        fused_decide_kernel<<<grid, ACC_THREADS, 0, st>>>(a, total_blocks);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        if ((e = launch_fp64_words(1, a, total_blocks, st)) != cudaSuccess) return e;
    }
    return accept_finish(a, total_blocks, st);
}

// Counts, offsets and output of an acceptance pass whose words and per-CTA
// counts are set.
static cudaError_t accept_finish(const AcceptArgs &a, int64_t total_blocks, cudaStream_t st) {
    accept_scan_kernel<<<a.n_segs, SCAN_THREADS, 0, st>>>(a);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || total_blocks == 0) return e;
    if (a.err != nullptr && a.out_lnl != nullptr) {
        // the ln L written out: FP64 for every output sample with a loose bound
        if ((e = cudaMemsetAsync(a.flag_count, 0, sizeof(unsigned long long), st)) != cudaSuccess)
            return e;
        accept_emit_kernel<true><<<(unsigned)total_blocks, ACC_THREADS, 0, st>>>(a);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        accept_fp64_list_kernel<2><<<152 * 4, 256, 0, st>>>(a, 0, 0);
        count_launch();
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    accept_emit_kernel<false><<<(unsigned)total_blocks, ACC_THREADS, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

}  // namespace joker
