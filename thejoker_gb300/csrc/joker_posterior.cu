// Per-sample FP64 work after the acceptance pass, one warp per sample (lanes
// over epochs):
//
// * the Gaussian posterior of the linear parameters of accepted samples --
//   the a and Ainv that CJokerHelper.likelihood_worker(1) builds
//   (thejoker/src/fast_likelihood.pyx:394-423, make_AAinv :255-297) and that
//   batch_get_posterior_samples (:471-545) hands to rng.multivariate_normal;
// * the unmarginalized ln-likelihood of full samples,
//   JokerSamples.ln_unmarginalized_likelihood (thejoker/samples.py:611-632):
//   the sum over epochs of ln N(y | K m(t) + trend(t), sigma^2 + s^2).
#include <cstdio>
#include "joker_fp64.cuh"

namespace joker {

// Posterior of the linear parameters of one sample.  With W = diag(w),
// G = Lambda^-1 + M W M^T and q = M W (y - M^T mu) (Acc64 with the jitter
// form), a = mu + G^-1 q, A = G^-1, and ln L from the same factorisation.
template <int L>
__device__ __noinline__ void posterior_one(const StarRec &st, const double *ep64, double P,
                                           double e, double om, double M0, double s, int k_clip,
                                           double *a_out, double *A_out, double *lnl_out) {
    Acc64<L, true> acc;
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
    if ((threadIdx.x & 31) != 0) return;
    double lam0 = st.lam0;
    if (st.k_scaled) {
        lam0 = st.sigK0sq / (1.0 - e * e) * pow(P / st.P0, -2.0 / 3.0);
        if (k_clip) lam0 = fmin(st.maxK2, lam0);
    }
    // G (full symmetric) and its LDL^T factorisation
    double G[L][L], D[L], Lw[L][L];
#pragma unroll
    for (int i = 0; i < L; ++i) {
#pragma unroll
        for (int k = 0; k <= i; ++k) { G[i][k] = acc.G[i][k]; G[k][i] = acc.G[i][k]; }
        G[i][i] += 1.0 / (i == 0 ? lam0 : st.lam[i]);
    }
    double logdetG = 0.0;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < L; ++k) {
        double dk = G[k][k];
#pragma unroll
        for (int m = 0; m < k; ++m) dk -= Lw[k][m] * Lw[k][m] * D[m];
        D[k] = dk;
        ok = ok && dk > 0.0;
        logdetG += log(dk);
#pragma unroll
        for (int i = k + 1; i < L; ++i) {
            double v = G[i][k];
#pragma unroll
            for (int m = 0; m < k; ++m) v -= Lw[i][m] * Lw[k][m] * D[m];
            Lw[i][k] = v / dk;
        }
    }
    // solve G x = b for b = q and for the unit vectors
    auto solve = [&](const double *b, double *x) {
        double z[L];
#pragma unroll
        for (int k = 0; k < L; ++k) {
            double v = b[k];
#pragma unroll
            for (int m = 0; m < k; ++m) v -= Lw[k][m] * z[m];
            z[k] = v;
        }
#pragma unroll
        for (int k = L - 1; k >= 0; --k) {
            double v = z[k] / D[k];
#pragma unroll
            for (int m = k + 1; m < L; ++m) v -= Lw[m][k] * x[m];
            x[k] = v;
        }
    };
    double x[L], quad = 0.0;
    solve(acc.q, x);
#pragma unroll
    for (int k = 0; k < L; ++k) {
        a_out[k] = ok ? st.mu[k] + x[k] : NAN;
        quad += acc.q[k] * x[k];
    }
#pragma unroll
    for (int c = 0; c < L; ++c) {
        double ec[L], col[L];
#pragma unroll
        for (int k = 0; k < L; ++k) ec[k] = k == c ? 1.0 : 0.0;
        solve(ec, col);
#pragma unroll
        for (int k = 0; k < L; ++k) A_out[k * L + c] = ok ? col[k] : NAN;
    }
    if (lnl_out)
        *lnl_out = ok ? -0.5 * (acc.rWr - quad + st.log_norm_rest + log(lam0) - acc.sum_log_w(st) + logdetG)
                      : INFINITY;
}

template <int L>
__global__ void __launch_bounds__(256) posterior_kernel(const StarRec *stars, const double *ep64,
                                                        int star, const double *P, const double *E,
                                                        const double *OM, const double *M0,
                                                        const double *S, int64_t stride,
                                                        const int64_t *rows, int64_t n, int jit,
                                                        int k_clip, double *a, double *A,
                                                        double *lnl) {
    const StarRec &st = stars[star];
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); i < n;
         i += nw) {
        const int64_t r = rows[i] * stride;
        posterior_one<L>(st, ep64, P[r], E[r], OM[r], M0[r], jit ? S[r] : 0.0, k_clip,
                         a + i * L, A + i * L * L, lnl ? lnl + i : nullptr);
    }
}

// ln of the unmarginalized likelihood: pars row = P, e, omega, M0, s, K, v_0..v_{nt-1}.
__global__ void __launch_bounds__(256) unmarginalized_kernel(const StarRec *stars,
                                                             const double *ep64, int star, int L,
                                                             const double *pars, int64_t n,
                                                             int nt, double dt_shift,
                                                             double *out) {
    const StarRec &st = stars[star];
    const int lane = threadIdx.x & 31;
    const int np = 6 + nt;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t i = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); i < n;
         i += nw) {
        const double *p = pars + i * np;
        const double P = p[0], e = p[1], om = p[2], M0 = p[3], s2 = p[4] * p[4], K = p[5];
        OrbitF64 orb;
        orb.init(P, e, om, M0);
        double acc = 0.0;
        const double *rec0 = ep64 + (size_t)st.epoch_off * REC64;
        for (int j = lane; j < st.n_epochs; j += 32) {
            const double *rec = rec0 + (size_t)j * REC64;
            const double dt = __ldg(rec) - dt_shift;
            // data velocity: y = y' + sum_{k>=1} mu_k T_k
            double y = __ldg(rec + 1);
            for (int k = 1; k < L; ++k) y += st.mu[k] * __ldg(rec + 2 + k);
            const double var = 1.0 / __ldg(rec + 2) + s2;
            const double m = orb.rv_unit(dt);
            // trend polynomial in (t - t_ref of the samples), Horner
            double tr = 0.0;
            for (int k = nt - 1; k >= 0; --k) tr = fma(tr, dt, p[6 + k]);
            const double d = fma(K, m, tr) - y;
            acc += -0.5 * (log(TWO_PI_D * var) + d * d / var);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) out[i] = acc;
    }
}

// rv[i * n_t + j] = K_i m_i(t_j - t0) for element rows (P, K, e, omega, M0):
// one thread per (orbit, time) pair.
__global__ void __launch_bounds__(256) rv_elements_kernel(const double *t, int n_t,
                                                          const double *el, int64_t n, double t0,
                                                          double *rv) {
    const int64_t total = n * n_t;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = g / n_t;
        const int j = (int)(g - i * n_t);
        const double *p = el + i * 5;
        OrbitF64 orb;
        orb.init(p[0], p[2], p[3], p[4]);
        rv[g] = p[1] * orb.rv_unit(t[j] - t0);
    }
}

cudaError_t launch_rv_elements(const double *t, int n_t, const double *el, int64_t n, double t0,
                               double *rv, cudaStream_t st) {
    const int64_t total = n * n_t;
    const int64_t blocks = (total + 255) / 256;
    const unsigned grid = (unsigned)(blocks < 152 * 16 ? blocks : 152 * 16);
    rv_elements_kernel<<<grid, 256, 0, st>>>(t, n_t, el, n, t0, rv);
    count_launch();
    return cudaGetLastError();
}

template <int L>
static cudaError_t launch_posterior_L(const StarRec *stars, const double *ep64, int star,
                                      const double *P, const double *E, const double *OM,
                                      const double *M0, const double *S, int64_t stride,
                                      const int64_t *rows, int64_t n, int jit, int k_clip,
                                      double *a, double *A, double *lnl, cudaStream_t st) {
    const int64_t warps = n < 152 * 8 * 4 ? n : 152 * 8 * 4;
    const unsigned grid = (unsigned)((warps + 7) / 8);
    posterior_kernel<L><<<grid, 256, 0, st>>>(stars, ep64, star, P, E, OM, M0, S, stride, rows,
                                              n, jit, k_clip, a, A, lnl);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_posterior(int L, const StarRec *stars, const double *ep64, int star,
                             const double *P, const double *E, const double *OM,
                             const double *M0, const double *S, int64_t stride,
                             const int64_t *rows, int64_t n, int jit, int k_clip, double *a,
                             double *A, double *lnl, cudaStream_t st) {
    switch (L) {
#define JOKER_POST_CASE(LL) \
        case LL: return launch_posterior_L<LL>(stars, ep64, star, P, E, OM, M0, S, stride, rows, \
                                               n, jit, k_clip, a, A, lnl, st);
        JOKER_POST_CASE(1) JOKER_POST_CASE(2) JOKER_POST_CASE(3)
        JOKER_POST_CASE(4) JOKER_POST_CASE(5) JOKER_POST_CASE(6)
#undef JOKER_POST_CASE
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_unmarginalized(const StarRec *stars, const double *ep64, int star, int L,
                                  const double *pars, int64_t n, int nt, double dt_shift,
                                  double *out, cudaStream_t st) {
    const int64_t warps = n < 152 * 8 * 4 ? n : 152 * 8 * 4;
    const unsigned grid = (unsigned)((warps + 7) / 8);
    unmarginalized_kernel<<<grid, 256, 0, st>>>(stars, ep64, star, L, pars, n, nt, dt_shift, out);
    count_launch();
    return cudaGetLastError();
}

}  // namespace joker

// ------------------------------------------------------------------ C ABI
namespace joker {
void set_last_error(const char *msg);
void stars_internals(const joker_stars *s, const StarRec **recs, const double **ep64,
                     const float **ep32, int *n_stars, int *L, int *jit, int **queue);
void cache_internals(const joker_cache *c, int64_t *cap, const double **P, const double **E,
                     const double **OM, const double **M0, const double **S, int64_t *stride,
                     const float4 **mx_a, const float4 **mx_b, const float **mx_s2);
}  // namespace joker

using namespace joker;

static int post_fail(int code, const char *msg) {
    set_last_error(msg);
    return code;
}

extern "C" int joker_linear_posterior(const joker_stars *stars, const joker_cache *cache,
                                      int star, const int64_t *d_rows, int64_t n, int k_clip,
                                      double *d_a, double *d_A, double *d_lnl, void *stream) {
    if (!stars || !cache) return post_fail(JOKER_EINVAL, "joker_linear_posterior: NULL handle");
    if (n < 0) return post_fail(JOKER_EINVAL, "joker_linear_posterior: n < 0");
    if (n == 0) return JOKER_OK;
    if (!d_rows || !d_a || !d_A)
        return post_fail(JOKER_EINVAL, "joker_linear_posterior: NULL device pointer");
    const StarRec *recs; const double *ep64; const float *ep32; int n_stars, L, jit; int *q;
    stars_internals(stars, &recs, &ep64, &ep32, &n_stars, &L, &jit, &q);
    if (star < 0 || star >= n_stars)
        return post_fail(JOKER_EINVAL, "joker_linear_posterior: star out of range");
    int64_t cap, stride; const double *P, *E, *OM, *M0, *S; const float4 *ma, *mb; const float *ms;
    cache_internals(cache, &cap, &P, &E, &OM, &M0, &S, &stride, &ma, &mb, &ms);
    const cudaError_t e = launch_posterior(L, recs, ep64, star, P, E, OM, M0, S, stride, d_rows,
                                           n, jit, k_clip, d_a, d_A, d_lnl, (cudaStream_t)stream);
    if (e != cudaSuccess) return post_fail(JOKER_ECUDA, cudaGetErrorString(e));
    return JOKER_OK;
}

extern "C" int joker_unmarginalized_lnl(const joker_stars *stars, int star, const double *d_pars,
                                        int64_t n, int n_trend, double dt_shift, double *d_out,
                                        void *stream) {
    if (!stars) return post_fail(JOKER_EINVAL, "joker_unmarginalized_lnl: NULL handle");
    if (n < 0 || n_trend < 1 || n_trend > JOKER_MAX_LINEAR - 1)
        return post_fail(JOKER_EINVAL, "joker_unmarginalized_lnl: bad n or n_trend");
    if (n == 0) return JOKER_OK;
    if (!d_pars || !d_out)
        return post_fail(JOKER_EINVAL, "joker_unmarginalized_lnl: NULL device pointer");
    const StarRec *recs; const double *ep64; const float *ep32; int n_stars, L, jit; int *q;
    stars_internals(stars, &recs, &ep64, &ep32, &n_stars, &L, &jit, &q);
    if (star < 0 || star >= n_stars)
        return post_fail(JOKER_EINVAL, "joker_unmarginalized_lnl: star out of range");
    const cudaError_t e = launch_unmarginalized(recs, ep64, star, L, d_pars, n, n_trend, dt_shift,
                                                d_out, (cudaStream_t)stream);
    if (e != cudaSuccess) return post_fail(JOKER_ECUDA, cudaGetErrorString(e));
    return JOKER_OK;
}

extern "C" int joker_rv_from_elements(const double *d_t, int n_t, const double *d_elems,
                                      int64_t n, double t0, double *d_rv, void *stream) {
    if (n < 0 || n_t < 0) return post_fail(JOKER_EINVAL, "joker_rv_from_elements: n < 0 or n_t < 0");
    if (n == 0 || n_t == 0) return JOKER_OK;
    if (!d_t || !d_elems || !d_rv)
        return post_fail(JOKER_EINVAL, "joker_rv_from_elements: NULL device pointer");
    const cudaError_t e = launch_rv_elements(d_t, n_t, d_elems, n, t0, d_rv, (cudaStream_t)stream);
    if (e != cudaSuccess) return post_fail(JOKER_ECUDA, cudaGetErrorString(e));
    return JOKER_OK;
}
