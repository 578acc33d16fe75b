// Internal types and device math shared by the kernels of libjoker_gb300.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>
#include "../../include/joker_gb300.h"

namespace joker {

constexpr int MAXL = JOKER_MAX_LINEAR;

// Host-side count of the kernels this library has launched (joker_launch_count).
void count_launch();
constexpr int TILE = 256;          // epochs staged in shared memory at a time
constexpr int REC32 = 20;          // floats per epoch record of the mixed kernel
constexpr int REC64 = 8;           // doubles per epoch record of the FP64 kernel
constexpr int MAX_CK = 8;          // early-exit checkpoints per star (fused pass)

// Per-star constants, built on the host in FP64 (joker_abi.cu).  Index 0 of
// the linear parameters is K; 1.. are v0, the offsets and the trend terms.
struct alignas(16) StarRec {
    int32_t epoch_off;     // first epoch in the packed per-epoch arrays
    int32_t n_epochs;
    int32_t k_scaled;      // FixedCompanionMass K prior
    int32_t pad;
    double mu0;            // K prior mean
    double lam0;           // K prior variance (not scaled)
    double sigK0sq;        // sigma_K0^2
    double P0;             // reference period of the scaled K prior
    double maxK2;          // max_K^2
    double log_kscale;     // log(sigma_K0^2 * P0^(2/3))
    double log_maxK2;      // log(max_K^2)
    // Sample-independent parts, jitter ignored.  With y'_n = y_n - sum_{j>=1}
    // mu_j T_jn, W = diag(ivar) and C = Lambda_T^-1 + T W T^T (the trend block):
    double chi2_0;              // y'^T W y' - c^T C^-1 c,  c = T W y'
    double logdet_const;        // N log 2pi - sum log ivar + sum_{j>=1} log lambda_j + log det C
    double cC[MAXL];            // C^-1 c          (entries 1..L-1)
    double Cinv[MAXL * MAXL];   // C^-1            (entries 1..L-1)
    // Jitter applied: everything is per sample.
    double lam[MAXL];           // prior variances (lam[0] = lam0)
    double mu[MAXL];            // prior means (mu[0] = mu0)
    double log_norm_rest;       // N log 2pi + sum_{j>=1} log lambda_j
    double sum_log_ivar;        // sum log ivar
    double ilam[MAXL];          // 1 / lambda_j (j >= 1; j = 0 when the K prior is not scaled)
    double iP0;                 // 1 / P0 of the scaled K prior
    // float-float copies for the mixed kernel's tail
    float chi2_0_hi, chi2_0_lo;
    float cC_hi[MAXL], cC_lo[MAXL];
    float Cinv_hi[MAXL * MAXL], Cinv_lo[MAXL * MAXL];
    float ilam_hi[MAXL], ilam_lo[MAXL];   // 1 / lambda_j (j >= 1)
    float sum_ivar;                        // sum ivar, bounds sum w under any jitter
    float mu0_f;
    int32_t mu0_zero;                      // mu0 == 0 (the usual K prior mean)
    int32_t pad2;
    // FP32-sum path (JOKER_MIXED_FAST).  With beta0 = C^-1 c the trend-only
    // fit, r_c = y' - T^T beta0 is the residual of that fit; words 18 and 19
    // of each REC32 epoch record hold r_c and ivar r_c as floats.
    float kappa_hi, kappa_lo;          // beta0^T Lambda_T^-1 beta0
    float ldc_hi, ldc_lo;              // logdet_const (jitter ignored)
    float lnr_hi, lnr_lo;              // log_norm_rest - sum log ivar (jitter applied)
    float Cn;                          // sum ivar r_c^2, rounded up
    float ivar_max;                    // max ivar, rounded up
    float Wjj[MAXL];                   // sum ivar T_j^2 (j >= 1), rounded up
    float log_kscale_f, log_maxK2_f;   // log_kscale, log_maxK2 rounded to float
    float log_lam0_f;                  // log lam0 rounded to float
    float phase_c;                     // 2 pi 2.5 2^-34 rms |t - t_ref| (ivar-weighted),
                                       // rounded up: the split phase's rounding per
                                       // unit of 1/P (radians), in the bound's norm
    // Early exit of the fused pass (L <= 3): after the first ck_k[c] epochs
    // the partial sums bound ln L from above.  Per checkpoint: P_j = sum over
    // those epochs of ivar r_c T_j minus (Lambda_T^-1 beta0)_j (j = 1, 2);
    // without jitter also C + kappa over those epochs, the inverse of the
    // partial trend block H (11, 12, 22) and log det H.
    int32_t n_ck;
    int32_t ck_k[MAX_CK];
    float ck[MAX_CK][8];          // P1, P2, C + kappa, Hi11, Hi12, Hi22, log det H, 0
    float ck_full[8];             // the same over all epochs (P = 0, C + kappa = chi2_0)
};

// One unit of the persistent likelihood kernels: `count` samples of star
// `star` starting at cache row `row0`; ln L goes to lnl[out_off + i].
struct alignas(16) WorkItem {
    int32_t star;
    int32_t count;
    int64_t row0;
    int64_t out_off;
    int32_t max_slot;
    int32_t pad;
};

struct LnlArgs {
    const StarRec *stars;
    const double *ep64;      // FP64 epoch records: [epoch][REC64]
    const float *ep32;       // mixed epoch records: [epoch][REC32]
    // FP64 sample columns (stride in doubles between consecutive samples)
    const double *P, *e, *om, *M0, *s;
    int64_t stride;
    // prepared mixed cache
    const float4 *mx_a;      // (1/P hi, 1/P lo, M0/2pi hi, M0/2pi lo)
    const float4 *mx_b;      // (e, cos w, sin w, log g) with g = P^(-2/3) / (1 - e^2)
    const float *mx_s2;      // s^2
    // Work items: explicit (items != nullptr) or implicit -- stars
    // [star0, star0 + n_sel) x rows [row0, row0 + count) in chunks of `chunk`,
    // star-major, stars visited in `order` (relative indices) when given.
    const WorkItem *items;
    int n_items;
    const int *n_items_dev;  // when set, the item count is read from device memory
    int star0, n_sel, chunk;
    int64_t row0, count, ld, ips;
    const int *order;
    int *queue;              // dynamic work counter, zeroed before launch
    double *lnl;
    unsigned long long *max_key;
    // mixed kernel only: per-sample error bound and the per-slot keys of
    // max(lnL + err) and max(lnL - err)
    float *err;
    unsigned long long *bound_key;   // [slot][2]
    float err_c0;                    // column-error constant of the bound
    // Fused first acceptance pass (FP32-sum kernel, implicit work items; NULL
    // fa_pcg: none).  Per slot the numpy PCG64 state and increment {state hi,
    // lo, inc hi, lo} before the slot's first uniform; the sample of row
    // row0 + j is number fa_first + j of the slot's stream (its uniform the
    // draw after fa_first + j steps).  Sample q of slot k is a candidate --
    // bit q % 32 of cand_words[k * cand_ld + q / 32] set -- unless its upper
    // bound lies below the running lower bound of the maximum by more than
    // -log u, which rejects it whatever the maximum.
    const unsigned long long *fa_pcg;
    int64_t fa_first;
    uint32_t *cand_words;
    int64_t cand_ld;
    // early exit (L <= 3): a warp stops evaluating epochs once the partial
    // sums put all its samples out of reach; their ln L is left at that upper
    // bound with an infinite error bound, and they get no candidate bit
    int fa_exit;
    // plain FP32-sum kernel only (L <= 3, or 4 without jitter): after the last
    // epoch a warp whose samples are all out of reach of the running lower
    // bound of the maximum (bound_key) stores their ln L in FP32 with an
    // infinite error bound, skipping the float-float tail; the acceptance
    // kernels reject such samples for every uniform
    int oor_tail;
};

// Largest work item (samples) of the fused pass: its per-pass generator
// states (one per 256 samples) are kept in shared memory.
constexpr int FUSED_MAX_CHUNK = 8192;

__device__ __forceinline__ int item_count(const LnlArgs &a) {
    return a.n_items_dev ? *((volatile const int *)a.n_items_dev) : a.n_items;
}

__device__ __forceinline__ WorkItem get_item(const LnlArgs &a, int it) {
    if (a.items) return a.items[it];
    WorkItem w;
    const int k = (int)(it / a.ips);
    const int64_t c = (int64_t)it - (int64_t)k * a.ips;
    const int sk = a.order ? a.order[k] : k;
    w.star = a.star0 + sk;
    w.row0 = a.row0 + c * a.chunk;
    const int64_t rem = a.count - c * a.chunk;
    w.count = (int)(rem < a.chunk ? rem : a.chunk);
    w.out_off = (int64_t)sk * a.ld + c * a.chunk;
    w.max_slot = sk;
    w.pad = 0;
    return w;
}

struct AcceptArgs {
    // refinement (mixed-precision ln L with per-sample error bounds); all NULL
    // for the plain pass
    const float *err;
    const unsigned long long *bound_key;   // [slot][2]: max(lnL + err), max(lnL - err)
    unsigned long long *exact_key;         // [slot]: exact FP64 maximum
    const StarRec *stars;
    const double *ep64;
    const float *ep32;                      // mixed epoch records (the float-float tier)
    float err_c0;                           // column-error constant of the mixed bound
    const double *P, *E, *OM, *M0, *S;
    int64_t stride;                         // doubles between consecutive samples (1 or 5)
    int L, jit;
    unsigned long long *n_refined;          // samples re-evaluated in FP64 (statistics)
    int write_max;                          // the maximum's FP64 pass writes its values back
                                            // to lnl (bound 0), sparing the decisions a
                                            // second evaluation of those samples
    uint32_t *amb_words;                    // undecided samples, one bit each (refinement)
    // flagged samples (max candidates, then undecided ones) compacted into a
    // list, (segment << 40) | index; entries past flag_cap fall back to
    // amb_words.  flag_count[0]: candidates, flag_count[1]: undecided.
    int64_t *flag_list;
    unsigned long long *flag_count;
    int64_t flag_cap;
    // candidate bits of the fused first pass: sample i of segment s at bit
    // i % 32 of cand_words[s * cand_ld + i / 32]
    const uint32_t *cand_words;
    int64_t cand_ld;
    const joker_accept_seg *segs;
    const int64_t *blk_base;     // n_segs + 1 prefix of CTA counts
    int64_t fixed_blocks;        // > 0: segment s owns CTA blocks [s * fixed, (s+1) * fixed)
    const int64_t *total_blocks_dev;  // when set: block count in device memory, kernels
                                      // loop over blocks (grid-stride), blk_base on device
    int n_segs;
    const double *lnl;
    const unsigned long long *max_key;
    int u_source;
    const double *u;
    uint32_t *words;             // accepted masks, one word per 32 samples
    int64_t *blk_count;          // per CTA accepted count, then its exclusive offset
    int64_t *out_idx;
    double *out_lnl;
    int64_t *count;
};

// ---------------------------------------------------------------- helpers
// Order-preserving key of a double from its bits (integer operations only).
__host__ __device__ __forceinline__ unsigned long long key_of_bits(long long b) {
    if ((b & 0x7FFFFFFFFFFFFFFFLL) > 0x7FF0000000000000LL)
        return 0xFFFFFFFFFFFFFFFFull;          // NaN dominates, as numpy's max
    return (b < 0) ? ~(unsigned long long)b : ((unsigned long long)b | 0x8000000000000000ull);
}

__host__ __device__ __forceinline__ unsigned long long double_to_key(double x) {
#ifdef __CUDA_ARCH__
    long long b = __double_as_longlong(x);
#else
    long long b; memcpy(&b, &x, 8);
#endif
    return key_of_bits(b);
}


__host__ __device__ __forceinline__ double key_to_double(unsigned long long k) {
    unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x; memcpy(&x, &b, 8); return x;
#endif
}

}  // namespace joker
