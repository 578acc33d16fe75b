/*
 * joker_gb300.h -- C ABI of the GB300 (sm_103a) marginal-likelihood and
 * rejection-sampling hot path of The Joker.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int status (JOKER_OK or one of the JOKER_E* codes below; never aborts) and,
 * for device work, a cudaStream_t passed as void*.  A failing call leaves a
 * one-line message readable through joker_last_error().
 *
 * Pointers named d_* are device pointers owned by the caller; every other
 * array argument is host memory, read during the call and not retained.
 *
 * Reference interfaces replaced (paths inside the adrn/thejoker project):
 *   joker_stars_create                    CJokerHelper.__init__
 *                                         thejoker/src/fast_likelihood.pyx:125-253
 *   joker_batch_marginal_ln_likelihood    CJokerHelper.batch_marginal_ln_likelihood
 *                                         thejoker/src/fast_likelihood.pyx:428-469
 *   joker_lnl                             the same loop over many stars and a
 *                                         shared prior cache (the pool map of
 *                                         marginal_ln_likelihood_worker,
 *                                         thejoker/multiproc_helpers.py:63-120)
 *   joker_accept                          exp(lls - lls.max()) > uu and the
 *                                         index list truncated to
 *                                         max_posterior_samples,
 *                                         thejoker/likelihood_helpers.py:107-109,
 *                                         thejoker/multiproc_helpers.py:256-258
 */
#ifndef JOKER_GB300_H
#define JOKER_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JOKER_ABI_VERSION 1

/* status codes */
#define JOKER_OK 0
#define JOKER_EINVAL 1      /* bad argument, shape or size */
#define JOKER_ECUDA 2       /* a CUDA runtime call failed */
#define JOKER_ENOMEM 3      /* device or host allocation failed */
#define JOKER_ERANGE 4      /* a size above a documented maximum */

/* limits */
#define JOKER_MAX_LINEAR 6  /* K + poly_trend + n_offsets */
#define JOKER_MIXED_LNL_TOL 1e-4  /* joker_accept_refined: |ln L - FP64 ln L| of every
                                     kept sample is at most this */

/* precision of the likelihood kernels */
#define JOKER_FP64 0        /* plain FP64 throughout */
#define JOKER_MIXED 1       /* FP64-accurate phase, FP32 Kepler, compensated
                               FP32 epoch sums, FP64 small solve; sin/cos of
                               the Kepler starter on the special-function unit */
#define JOKER_MIXED_ACCURATE 2  /* as JOKER_MIXED with correctly rounded sincosf */
#define JOKER_MIXED_FP64_TAIL 3 /* as JOKER_MIXED with the per-sample solve in FP64
                                   instead of float-float (no error bound) */
#define JOKER_MIXED_FAST 4      /* the first pass of the refined acceptance: FP32
                                   epoch sums re-centred on each star's trend-only
                                   fit, float-float solve, and a rigorous
                                   per-sample bound (looser than JOKER_MIXED's);
                                   more than three linear parameters with the
                                   jitter applied run as JOKER_MIXED */

/* jitter handling (the reference Cython computes the jittered inverse variance
   but never reads it, fast_likelihood.pyx:458; its NumPy test oracle applies
   it, thejoker/src/tests/py_likelihood.py:168-170) */
#define JOKER_JITTER_REFERENCE 0   /* s ignored, as CJokerHelper */
#define JOKER_JITTER_APPLIED 1     /* ivar / (1 + s^2 ivar) per sample */

/* source of the acceptance uniforms */
#define JOKER_U_ARRAY 0     /* d_u[u_off + i] */
#define JOKER_U_PCG64 1     /* numpy PCG64 stream, reproduced on the device */

typedef struct joker_stars joker_stars;   /* opaque, device-resident star table */
typedef struct joker_cache joker_cache;   /* opaque, device-resident prior cache */

/* One segment of the acceptance pass: the ln L values of one star over a
 * contiguous run of samples, the uniforms to test them against, and where the
 * accepted indices go.  Plain C layout, 96 bytes. */
typedef struct {
    int64_t lnl_off;       /* first ln L of the segment in d_lnl */
    int64_t n;             /* number of samples */
    int64_t idx_base;      /* added to the in-segment position of each accepted sample */
    int64_t out_off;       /* first output slot in d_out_idx / d_out_lnl */
    int64_t max_out;       /* output capacity; acceptance beyond it is counted, not written */
    int64_t u_off;         /* JOKER_U_ARRAY: first uniform in d_u */
    uint64_t pcg_state_hi; /* JOKER_U_PCG64: PCG64 state and increment, positioned */
    uint64_t pcg_state_lo; /*   so that the next draw is the segment's first uniform */
    uint64_t pcg_inc_hi;
    uint64_t pcg_inc_lo;
    int32_t max_slot;      /* which running maximum (d_max_key) the segment uses */
    int32_t star;          /* joker_accept_refined: the segment's star */
    int64_t row0;          /* joker_accept_refined: cache row of the segment's sample 0 */
} joker_accept_seg;

int joker_abi_version(void);
const char *joker_last_error(void);
/* Kernels this library has launched since it was loaded, counted on the host
 * at each launch (all devices, all threads).  A CUDA graph that captured
 * launches replays them without counting.  No counterpart in the reference. */
uint64_t joker_launch_count(void);

/* ---- star table -----------------------------------------------------------
 * Mirrors CJokerHelper.__init__ (fast_likelihood.pyx:125-253) for n_stars
 * stars at once.  Star k owns epochs [epoch_offsets[k], epoch_offsets[k+1]).
 *   t, rv, ivar     times (days), velocities and inverse variances per epoch
 *   t_ref           reference time per star (the reference's _t_ref_bmjd)
 *   trend_M         total_epochs x (n_linear-1), row-major: the columns of
 *                   CJokerHelper's trend_M (v0 / offset indicators, then
 *                   (t - t_ref)^k), fast_likelihood.pyx:174-184
 *   mu, lambda      n_stars x n_linear prior means / variances in the
 *                   CJokerHelper index order K, v0, offsets..., v1, ...
 *   k_prior         n_stars x 4: {scaled, sigma_K0, P0, max_K}; scaled != 0 is
 *                   the FixedCompanionMass prior (the reference's
 *                   fixed_K_prior == 0, :225-228, :461-464), whose variance
 *                   min(max_K^2, sigma_K0^2 / (1 - e^2) (P / P0)^(-2/3))
 *                   replaces lambda[k][0] per sample
 *   jitter_mode     JOKER_JITTER_REFERENCE or JOKER_JITTER_APPLIED
 * Errors: JOKER_EINVAL for n_linear outside [1, JOKER_MAX_LINEAR], a star
 * without epochs, non-increasing offsets or a non-positive ivar or lambda. */
int joker_stars_create(joker_stars **out, int n_stars, int n_linear,
                       const int64_t *epoch_offsets, const double *t,
                       const double *rv, const double *ivar, const double *t_ref,
                       const double *trend_M, const double *mu,
                       const double *lambda, const double *k_prior,
                       int jitter_mode);
int joker_stars_destroy(joker_stars *stars);

/* A table of n_slots empty stars with room for max_epochs epochs each, for a
 * serving loop that takes stars as they arrive.  joker_stars_set fills (or
 * refills) one slot with the per-star arguments of joker_stars_create; its
 * copies are ordered on `stream`. */
int joker_stars_create_slots(joker_stars **out, int n_slots, int max_epochs, int n_linear,
                             int jitter_mode);
int joker_stars_set(joker_stars *stars, int slot, int n_epochs, const double *t,
                    const double *rv, const double *ivar, double t_ref, const double *trend_M,
                    const double *mu, const double *lambda, const double *k_prior,
                    void *stream);
int joker_stars_info(const joker_stars *stars, int *n_stars, int *n_linear,
                     int64_t *total_epochs, int *max_epochs);

/* ---- prior cache ----------------------------------------------------------
 * A device-resident copy of packed prior samples (JokerSamples.pack order
 * P, e, omega, M0, s in internal units, thejoker/samples.py:404-445) kept both
 * as FP64 columns and in the prepared form the mixed kernel reads.
 * joker_cache_load converts rows [row0, row0 + n) from a device n x 5
 * row-major FP64 array; it rejects e outside [0, 1) or P <= 0 lazily (the
 * result for such rows is NaN, as the reference's arithmetic would give). */
int joker_cache_create(joker_cache **out, int64_t capacity);
int joker_cache_destroy(joker_cache *cache);
/* A cache over the caller's packed (n, 5) FP64 chunk without a copy: the
 * FP64 columns alias the chunk and the mixed kernel prepares each sample in
 * registers (the values equal those of joker_cache_load).  The chunk may be
 * device memory or pinned host memory (read through its mapped device
 * address, 40 bytes per sample per ln L call over the host link); it must
 * outlive the view.  joker_cache_load on a view returns JOKER_EINVAL.
 * Replaces the staging of batch_marginal_ln_likelihood's chunk
 * (fast_likelihood.pyx:428-451) for callers that keep it pinned. */
int joker_cache_create_view(joker_cache **out, const double *chunk, int64_t n);
/* The same view over five separate FP64 columns of n samples each (P, e,
 * omega, M0, s in the reference's internal units), for callers that hold
 * the prior samples column by column (JokerSamples keeps one array per
 * parameter, samples.py:404-445, which pack() interleaves into the chunk of
 * fast_likelihood.pyx:428).  Each column may be device memory or pinned host
 * memory and must outlive the view; s is read only with the jitter applied
 * but must be given. */
int joker_cache_bind(joker_cache **out, const double *P, const double *e, const double *omega,
                     const double *M0, const double *s, int64_t n);
int joker_cache_load(joker_cache *cache, const double *d_chunk, int64_t n,
                     int64_t row0, void *stream);
int64_t joker_cache_capacity(const joker_cache *cache);

/* ---- likelihood -----------------------------------------------------------
 * Drop-in for CJokerHelper.batch_marginal_ln_likelihood on star `star`:
 * d_chunk is n_samples x 5 row-major FP64 (the reference's chunk, :428-451),
 * d_lnl receives n_samples FP64 ln L values computed in FP64. */
int joker_batch_marginal_ln_likelihood(const joker_stars *stars, int star,
                                       const double *d_chunk, int64_t n_samples,
                                       double *d_lnl, void *stream);

/* ln L of stars [star0, star0 + n_sel) over cache rows [row0, row0 + count).
 * d_lnl is n_sel x count with row stride ld.  When d_max_key is not NULL,
 * d_max_key[k] holds an order-preserving integer image of the running
 * maximum of star star0+k and is raised atomically (it must be zeroed, or hold
 * a previous maximum, before the call).  precision: JOKER_FP64, JOKER_MIXED,
 * JOKER_MIXED_ACCURATE, JOKER_MIXED_FP64_TAIL or JOKER_MIXED_FAST.
 * Mixed precisions only: d_err (optional, laid out like d_lnl) receives a
 * bound on |lnL - lnL_FP64| per sample, and d_bound_key (optional, 2 per star)
 * the running maxima of lnL + err and lnL - err.
 * block (threads per CTA, 0 = 128) and chunk (samples per work item, a
 * multiple of block, 0 = 1024) tune the launch.  Calls that share one
 * joker_stars handle must be ordered on one stream. */
int joker_lnl(const joker_stars *stars, const joker_cache *cache, int star0,
              int n_sel, int64_t row0, int64_t count, int precision,
              double *d_lnl, int64_t ld, uint64_t *d_max_key, float *d_err,
              uint64_t *d_bound_key, int block, int64_t chunk, void *stream);

/* Decode an order-preserving key back to the double it encodes. */
double joker_key_to_double(uint64_t key);

/* ---- acceptance -----------------------------------------------------------
 * For each segment: keep_i = exp(lnl_i - max) > u_i with max the decoded
 * d_max_key[seg.max_slot]; the indices (idx_base + i) of kept samples are
 * written in ascending order to d_out_idx[out_off ...] (at most max_out of
 * them), their ln L to d_out_lnl (if not NULL), and the total number kept to
 * d_count[segment].  segs is a host array of n_segs segments.  d_work must
 * hold joker_accept_workspace(segs, n_segs) bytes. */
int64_t joker_accept_workspace(const joker_accept_seg *segs, int n_segs);
int joker_accept(const joker_accept_seg *segs, int n_segs, const double *d_lnl,
                 const uint64_t *d_max_key, int u_source, const double *d_u,
                 int64_t *d_out_idx, double *d_out_lnl, int64_t *d_count,
                 void *d_work, int64_t work_bytes, void *stream);

/* The acceptance pass over mixed-precision ln L values with their error
 * bounds (d_err, d_bound_key from joker_lnl), exact with respect to FP64:
 * the maximum is re-evaluated in FP64 among the samples whose interval can
 * reach it, and every sample whose decision the interval leaves open is
 * re-evaluated in FP64 from the cache (seg.star, seg.row0 locate it).  The
 * kept indices are then those the FP64 path would keep.  d_exact_key (one per
 * max_slot) receives the FP64 maxima -- or, with max_given != 0, already holds
 * them (from joker_refine_max, e.g. combined over ranks that each own a range
 * of the same star's samples).  d_n_refined (optional) counts the re-evaluated
 * samples.  When d_out_lnl is given, every kept sample written out (the first
 * max_out of a segment) whose bound exceeds JOKER_MIXED_LNL_TOL is
 * re-evaluated as well, so every ln L in d_out_lnl is within that of the FP64
 * value.  Each re-evaluated sample's FP64 ln L is written back to d_lnl
 * and its bound in d_err set to 0.  Same workspace as joker_accept. */
int joker_accept_refined(const joker_stars *stars, const joker_cache *cache,
                         const joker_accept_seg *segs, int n_segs, double *d_lnl,
                         float *d_err, const uint64_t *d_bound_key,
                         uint64_t *d_exact_key, int n_slots, int max_given, int u_source,
                         const double *d_u, int64_t *d_out_idx, double *d_out_lnl,
                         int64_t *d_count, uint64_t *d_n_refined, void *d_work,
                         int64_t work_bytes, void *stream);

/* The first step of joker_accept_refined alone: raise d_exact_key[slot] to the
 * FP64 maximum over the samples of the segments whose interval
 * [lnL - err, lnL + err] reaches the slot's largest lower bound (d_bound_key).
 * d_exact_key must be zeroed (or hold a smaller maximum) before the call. */
int joker_refine_max(const joker_stars *stars, const joker_cache *cache,
                     const joker_accept_seg *segs, int n_segs, const double *d_lnl,
                     const float *d_err, const uint64_t *d_bound_key, uint64_t *d_exact_key,
                     uint64_t *d_n_refined, void *d_work, int64_t work_bytes, void *stream);

/* The band refinement of mixed-precision ln L values (no counterpart in the
 * reference, whose values are all FP64): every sample of the segments whose
 * interval [lnL - err, lnL + err] reaches within `band` of its slot's FP64
 * maximum d_exact_key[seg.max_slot] (from joker_refine_max or
 * joker_accept_refined), and whose bound err exceeds `tol`, is re-evaluated
 * in FP64; its FP64 ln L is written to d_lnl and its bound set to 0.  Samples
 * without a finite value or bound are re-evaluated too.  Afterwards every
 * ln L of the segments within `band` of the maximum is within `tol` of the
 * FP64 path's value; below the band each value keeps its mixed bound.  The
 * host mirror uses band = JOKER_MIXED_LNL_BAND and tol = JOKER_MIXED_LNL_TOL
 * for the ln L values it returns (marginal_ln_likelihood,
 * thejoker/thejoker.py:93-138; return_all_logprobs, :140-257).  Same
 * workspace as joker_accept. */
#define JOKER_MIXED_LNL_BAND 40.0  /* nats: exp(-40) < 2^-53, below any nonzero
                                      uniform of the acceptance test */
int joker_refine_band(const joker_stars *stars, const joker_cache *cache,
                      const joker_accept_seg *segs, int n_segs, double *d_lnl, float *d_err,
                      const uint64_t *d_exact_key, double band, double tol,
                      uint64_t *d_n_refined, void *d_work, int64_t work_bytes, void *stream);

/* ---- fused first acceptance pass (JOKER_MIXED_FAST) -------------------------
 * joker_lnl_fused is joker_lnl at JOKER_MIXED_FAST with the first pass of the
 * acceptance folded into the ln L kernel: each sample's uniform is drawn from
 * its star's numpy PCG64 stream inside the kernel, and every sample that the
 * running bounds cannot reject -- whatever the maximum turns out to be -- gets
 * a candidate bit.  joker_accept_fused then finds the FP64 maxima among the
 * candidates and decides them; a sample without the bit is rejected.  The
 * two calls keep exactly the rows joker_lnl + joker_accept_refined keep
 * (the FP64 decisions), without the two full scans over ln L and its bounds.
 *
 * joker_lnl_fused: d_pcg (device, n_sel x 4 {state_hi, state_lo, inc_hi,
 * inc_lo}) holds each star's generator before its first uniform; row row0 + j
 * is sample number first + j of the star's stream (its uniform the draw after
 * first + j steps; first a multiple of 32, as for a slice of a larger run).
 * Sample q of star star0 + k gets bit q % 32 of d_cand[k * cand_ld + q / 32]
 * (cand_ld >= (first + count + 31) / 32 words); the other bits of the words
 * it covers are written, words outside [first, first + count) are not.
 * d_err and d_bound_key are required (zeroed, or holding smaller maxima,
 * before the first call of a run); chunk a multiple of 128 and at most 8192
 * (0 = 1024).  A jittered table with more than three linear parameters
 * returns JOKER_EINVAL (use joker_lnl + joker_accept_refined).
 * With at most three linear parameters, a warp of 64 samples whose ln L all
 * lie more than 746 nats below the running lower bound of the maximum after
 * the last epoch (rejected for every uniform, and none the maximum) keeps
 * their ln L in FP32 with d_err +infinity, skipping the float-float tail and
 * its bound; every other sample gets its usual value and bound.
 * early_exit != 0 (at most three linear parameters; ignored otherwise): a
 * warp also stops evaluating epochs at a checkpoint (after 8, 12, 16, 24,
 * 32, 48, 64 or 96 epochs, stars of at most 256 epochs) once the partial
 * sums put every one of its samples that far below; those samples' d_lnl
 * holds that upper bound and d_err +infinity.  joker_accept_fused keeps the
 * same rows either way.  No counterpart in the reference, which evaluates
 * every sample in full.
 *
 * joker_accept_fused: joker_accept_refined's output contract for segments
 * whose candidate bits segment s finds at d_cand + s * cand_ld (sample i at
 * bit i % 32 of word i / 32; cand_ld a multiple of 4, d_cand 16-byte
 * aligned), uniforms from the segments' PCG64 states (u_source
 * JOKER_U_PCG64).  d_exact_key (n_slots) receives the FP64 maxima.
 * Same workspace as joker_accept.
 * Replace, as joker_lnl + joker_accept_refined do, the ln L loop and the
 * acceptance of rejection_sample (thejoker/likelihood_helpers.py:40-66,
 * 107-109). */
int joker_lnl_fused(const joker_stars *stars, const joker_cache *cache, int star0, int n_sel,
                    int64_t row0, int64_t count, const uint64_t *d_pcg, int64_t first,
                    double *d_lnl, int64_t ld, uint64_t *d_max_key, float *d_err,
                    uint64_t *d_bound_key, uint32_t *d_cand, int64_t cand_ld, int64_t chunk,
                    int early_exit, void *stream);
int joker_accept_fused(const joker_stars *stars, const joker_cache *cache,
                       const joker_accept_seg *segs, int n_segs, double *d_lnl, float *d_err,
                       const uint64_t *d_bound_key, uint64_t *d_exact_key, int n_slots,
                       const uint32_t *d_cand, int64_t cand_ld, int64_t *d_out_idx,
                       double *d_out_lnl, int64_t *d_count, uint64_t *d_n_refined,
                       void *d_work, int64_t work_bytes, void *stream);

/* ---- iterative rejection, one device-resident round at a time --------------
 * Replaces the loop of iterative_rejection_inmem
 * (thejoker/likelihood_helpers.py:130-229) for every star of a joker_stars
 * table at once, over library rows [lib_row0, lib_row0 + lib_size) of the
 * cache.  Per star: init_batch samples first (growth_factor * n_requested in
 * the reference), then n_process = int(safety_factor * n_need / n_good *
 * n_evals) clamped to the library; every round draws fresh uniforms for the
 * whole prefix from the star's numpy PCG64 stream (pcg_states: n_stars x 4
 * uint64 -- state hi, lo, increment hi, lo -- positioned at its next draw);
 * a star stops when n_good >= n_requested, when the library is exhausted, on
 * zero accepted samples, or after maxiter rounds.  precision: JOKER_FP64, or
 * JOKER_MIXED / JOKER_MIXED_ACCURATE with the acceptance refined to the FP64
 * decisions.  joker_iter_round launches one round without host copies,
 * allocation or synchronisation, so a round can be captured in a CUDA graph
 * and replayed until the finished-star count (joker_iter_outputs) reaches
 * n_stars.  A handle allocates its buffers once, at creation. */
typedef struct joker_iter joker_iter;
int joker_iter_create(joker_iter **out, const joker_stars *stars, const joker_cache *cache,
                      int precision, int64_t lib_row0, int64_t lib_size, int n_requested,
                      int64_t init_batch, double safety_factor, int maxiter,
                      const uint64_t *pcg_states, int chunk);
int joker_iter_destroy(joker_iter *it);
int joker_iter_round(joker_iter *it, void *stream);
int joker_iter_outputs(const joker_iter *it, int64_t **d_state, int64_t **d_idx,
                       double **d_lnl, int **d_done, uint64_t **d_n_refined);
/* A handle with every slot of a slot table empty, whose per-star ln L
 * buffers are carved from one pool of pool_samples samples, and the
 * admission of one request into a slot between rounds: its library budget
 * (cache rows [lib_row0, lib_row0 + budget)), samples requested (at most
 * max_requested), first batch, pool offset and PCG64 state.  A slot is free
 * again once its state row reports done != 0; admitting into it takes it out
 * of the finished-star count.  joker_iter_admit also restarts a star of a
 * joker_iter_create handle (same slot, its own pool range). */
int joker_iter_create_pool(joker_iter **out, const joker_stars *stars, const joker_cache *cache,
                           int precision, int64_t lib_row0, int64_t pool_samples,
                           int max_requested, double safety_factor, int maxiter, int chunk);
int joker_iter_admit(joker_iter *it, int slot, int64_t budget, int n_requested,
                     int64_t init_batch, int64_t pool_off, const uint64_t *pcg_state,
                     void *stream);
/* Samples evaluated per round over all stars (0, the default: no limit).  A
 * star whose batch is larger than its equal share of the budget spreads the
 * batch over several rounds; its acceptance runs once the batch is complete,
 * so the results do not depend on the budget, only the time a round takes.
 * Read at joker_iter_round launch: a captured graph keeps the budget it was
 * captured with.  No counterpart in the reference. */
int joker_iter_set_round_budget(joker_iter *it, int64_t samples);
/* Synchronous copy of the same outputs to host arrays (any may be NULL). */
int joker_iter_read(const joker_iter *it, int64_t *h_state, int64_t *h_idx, double *h_lnl,
                    int *h_done, uint64_t *h_n_refined);
/* Asynchronous copies on `stream`: the state table (n_stars x 8, when h_state
 * is not NULL) and the index rows (max_requested each) of the n_slots slots
 * listed in `slots` (host array), row k to h_idx[k * max_requested ...].  Host
 * buffers should be pinned for the copies to overlap device work; the caller
 * synchronises with the stream before reading them.  A serving loop reads the
 * small state table after every round and only the finished slots' rows.  No
 * counterpart in the reference. */
int joker_iter_read_async(const joker_iter *it, int64_t *h_state, const int *slots, int n_slots,
                          int64_t *h_idx, void *stream);

/* ---- prior samples on the device ------------------------------------------
 * The producer of the prior cache (JokerPrior.sample, thejoker/prior.py
 * :297-407; UniformLog and Kipping13Global, thejoker/distributions.py:19-28,
 * 171-176): n samples of the default prior's nonlinear parameters drawn on
 * the device into cache rows [row0, row0 + n) (FP64 columns and the mixed
 * kernel's prepared form), and into d_packed (n x 5, P e omega M0 s) when not
 * NULL.  Sample g = first_index + i depends only on (seed, g): Philox4x32-10
 * counters (g, block) under the 64-bit seed.  P ~ log-uniform(P_min, P_max),
 * e ~ Beta(e_alpha, e_beta), omega and M0 ~ U[0, 2 pi), s fixed or
 * log-normal.  The draws follow these distributions, not numpy's streams.
 * JOKER_ERANGE if a gamma rejection loop ran out of tries for some sample
 * (its e is clamped to [0, 1)); JOKER_EINVAL for a bad spec or a cache view. */
#define JOKER_S_FIXED 0
#define JOKER_S_LOGNORMAL 1
typedef struct {
    double P_min, P_max;     /* days, 0 < P_min < P_max */
    double e_alpha, e_beta;  /* Beta shape parameters, > 0 */
    int32_t s_kind;          /* JOKER_S_FIXED or JOKER_S_LOGNORMAL */
    int32_t pad;
    double s_value;          /* JOKER_S_FIXED: s */
    double s_mu, s_sigma;    /* JOKER_S_LOGNORMAL: ln s ~ N(s_mu, s_sigma) */
} joker_prior_spec;
int joker_prior_sample(joker_cache *cache, int64_t row0, int64_t n, const joker_prior_spec *spec,
                       uint64_t seed, int64_t first_index, double *d_packed, void *stream);

/* ---- after acceptance ----------------------------------------------------
 * joker_linear_posterior: for the n cache rows d_rows[i] (device array) of
 * star `star`, the Gaussian posterior of the linear parameters (K, v0,
 * offsets, trend terms; the CJokerHelper order) -- mean d_a[i*L + k] and
 * covariance d_A[i*L*L + k*L + j] = (Ainv^-1)[k][j] -- and ln L of the sample
 * (d_lnl, may be NULL; +inf where Ainv is not positive definite, with NaN a
 * and A), in FP64.  These are the a and inv(Ainv) that
 * CJokerHelper.batch_get_posterior_samples passes to rng.multivariate_normal
 * (fast_likelihood.pyx:394-423, :519-530).  k_clip = 0 uses the scaled K
 * prior variance without the max_K clip, as batch_get_posterior_samples does
 * (:519-521); 1 clips it as batch_marginal_ln_likelihood does.  Jitter per the
 * star table's jitter_mode.
 *
 * joker_unmarginalized_lnl: ln of the unmarginalized likelihood of n full
 * samples (JokerSamples.ln_unmarginalized_likelihood, samples.py:611-632):
 * sum over the star's epochs of ln N(y | K m(t) + sum_k v_k (t - t_ref')^k,
 * sigma^2 + s^2).  d_pars: n x (6 + n_trend) row-major FP64 rows
 * P, e, omega, M0, s, K, v_0 .. v_{n_trend-1} (internal units);
 * dt_shift = t_ref' - t_ref of the star's data (days), t_ref' being the
 * samples' reference time.  Offsets are not part of the model, as in the
 * reference's JokerSamples.get_orbit. */
int joker_linear_posterior(const joker_stars *stars, const joker_cache *cache, int star,
                           const int64_t *d_rows, int64_t n, int k_clip, double *d_a,
                           double *d_A, double *d_lnl, void *stream);
int joker_unmarginalized_lnl(const joker_stars *stars, int star, const double *d_pars, int64_t n,
                             int n_trend, double dt_shift, double *d_out, void *stream);

/* ---- radial velocity of Keplerian orbits ---------------------------------
 * Replaces twobody's c_rv_from_elements(t, rv, N_t, P, K, e, omega, phi0,
 * t0, tol, maxiter) as bound at thejoker/src/fast_likelihood.pyx:27-30 and
 * called at :453-455, batched over n element sets on the device:
 *   d_rv[i * n_t + j] = K_i (cos(omega_i + f_ij) + e_i cos omega_i),
 *   M_ij = 2 pi (d_t[j] - t0) / P_i - M0_i,
 * f the true anomaly.  d_elems: n x 5 row-major FP64 rows (P, K, e, omega,
 * M0), 0 <= e < 1.  The FP64 solver is the one the ln L kernels use
 * (non-iterative, converged to FP64), so tol and maxiter have no
 * counterpart.  All pointers are device pointers. */
int joker_rv_from_elements(const double *d_t, int n_t, const double *d_elems, int64_t n,
                           double t0, double *d_rv, void *stream);

/* ---- one-call rejection step ----------------------------------------------
 * For stars [star0, star0 + n_sel) over cache rows [row0, row0 + count): the
 * ln L of every (star, sample) at `precision`, each star's maximum, and the
 * acceptance exp(lnl - max) > u against the star's numpy PCG64 stream (pcg:
 * n_sel x 4 {state_hi, state_lo, inc_hi, inc_lo}, positioned so that the
 * next draw is the uniform of row row0), refined to the FP64 decisions for
 * the mixed precisions.  Star k's kept cache rows go to d_out_idx[k * max_out
 * ...] (ascending, at most max_out), their ln L to d_out_lnl (optional), the
 * number kept to d_count[k].  d_work: joker_rejection_workspace(n_sel,
 * count, max_out, precision) bytes of device memory, 256-byte aligned.
 * Replaces, for a batch of stars, marginal_ln_likelihood_inmem plus the
 * acceptance of rejection_sample (thejoker/likelihood_helpers.py:40-66,
 * 107-109; thejoker/multiproc_helpers.py:63-120, 256-258): the sequence
 * joker_lnl + joker_accept / joker_accept_refined in one call -- for
 * JOKER_MIXED_FAST, joker_lnl_fused + joker_accept_fused (the workspace then
 * also holds the generator states and the candidate bits). */
int64_t joker_rejection_workspace(int n_sel, int64_t count, int64_t max_out, int precision);
int joker_rejection_sample(const joker_stars *stars, const joker_cache *cache, int star0,
                           int n_sel, int64_t row0, int64_t count, int precision,
                           const uint64_t *pcg, int64_t max_out, int64_t *d_out_idx,
                           double *d_out_lnl, int64_t *d_count, void *d_work,
                           int64_t work_bytes, void *stream);

/* ---- acceptance without allocation ---------------------------------------
 * No counterpart in the reference.  joker_accept_noalloc is joker_accept for
 * callers that must not allocate device memory: a serving loop with
 * per-request deadlines (cudaMalloc may synchronise the device and has
 * unbounded latency), or a plugin inside a host framework whose caching
 * allocator already holds the device's free memory.  It needs no workspace.
 * Its scratch space is one fixed array of 2,220,288 bytes inside the
 * library.  Limits: at most JOKER_NOALLOC_MAX_SEGS segments and
 * JOKER_NOALLOC_MAX_BLOCKS blocks of 8192 samples (each segment rounded up;
 * about 2^24 samples in all); larger calls return JOKER_ERANGE.  All calls
 * share the array: calls that overlap on the GPU (another stream, another
 * host thread) race and must not be issued.
 * Set-up: the first call on a device, with that device current, looks up the
 * array's address and loads the pass's kernels; under lazy module loading
 * (the CUDA default) that is also when the device's copy of the array is
 * allocated.  Make that first call at start-up, before any stream capture: a
 * call with n_segs = 0 does the set-up and nothing else.  After it the device
 * holds the array until the process exits, and no call allocates: no
 * cudaMalloc, cudaFree or heap use.  The address is kept for the life of the
 * process, so the entry point must not be used on a device after
 * cudaDeviceReset of that device.
 * segs is copied to the device on `stream`: from pageable memory before the
 * call returns; from pinned memory later, so pinned segs must stay unchanged
 * until the stream has passed the call.  Because every call copies from host
 * memory (segs and a block table on the stack), no call may be captured
 * into a CUDA graph. */
#define JOKER_NOALLOC_MAX_SEGS 1024
#define JOKER_NOALLOC_MAX_BLOCKS 2048
int joker_accept_noalloc(const joker_accept_seg *segs, int n_segs, const double *d_lnl,
                         const uint64_t *d_max_key, int u_source, const double *d_u,
                         int64_t *d_out_idx, double *d_out_lnl, int64_t *d_count,
                         void *stream);

#ifdef __cplusplus
}
#endif
#endif /* JOKER_GB300_H */
