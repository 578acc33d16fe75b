// C ABI of libjoker_gb300 (declared in include/joker_gb300.h): handle
// management, the per-star FP64 preparation done once on the host, and the
// launchers.  No torch types cross this boundary.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include "joker_internal.cuh"

namespace joker {
cudaError_t launch_lnl(int precision, int L, bool jit, const LnlArgs &a, int block,
                       cudaStream_t st);
cudaError_t launch_prepare(const double *chunk, int64_t n, int64_t row0, double *P, double *E,
                           double *OM, double *M0, double *S, float4 *mx_a, float4 *mx_b,
                           float *mx_s2, cudaStream_t st);
cudaError_t launch_accept(const AcceptArgs &a, int64_t total_blocks, cudaStream_t st,
                          bool max_given = false);
cudaError_t launch_refine_max(const AcceptArgs &a, int64_t total_blocks, cudaStream_t st);
cudaError_t launch_refine_band(const AcceptArgs &a, int64_t total_blocks, double band, float tol,
                               cudaStream_t st);
int64_t accept_blocks(const joker_accept_seg *segs, int n_segs, int64_t *blk_base_host);
}  // namespace joker

using namespace joker;

static thread_local std::string g_err;

static int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CUDA_TRY(expr)                                                                     \
    do {                                                                                   \
        cudaError_t e_ = (expr);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return fail(JOKER_ECUDA, "%s: %s", #expr, cudaGetErrorString(e_));             \
    } while (0)

struct joker_stars {
    int n_stars = 0, L = 0, jitter = 0, max_epochs = 0;
    int slot_epochs = 0;         // > 0 for a slot table (joker_stars_create_slots)
    int64_t total_epochs = 0;
    std::vector<int64_t> off;
    StarRec *d_stars = nullptr;
    double *d_ep64 = nullptr;
    float *d_ep32 = nullptr;
    int *d_queue = nullptr;
    int *d_order = nullptr;      // stars sorted by epoch count, largest first
};

struct joker_cache {
    int64_t cap = 0;
    double *P = nullptr, *E = nullptr, *OM = nullptr, *M0 = nullptr, *S = nullptr;
    int64_t stride = 1;          // 5 for a view over a packed chunk
    bool view = false;           // FP64 columns alias the caller's chunk; no prepared form
    float4 *mx_a = nullptr, *mx_b = nullptr;
    float *mx_s2 = nullptr;
    int *flag = nullptr;         // device word for joker_prior_sample's status
};

namespace joker {
// lets the other translation units report through joker_last_error()
void set_last_error(const char *msg) { g_err = msg; }

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// Grid size of a persistent launch on the current device: SM count x resident
// CTAs of `kern` at `block` threads.  Both are looked up once per (device,
// kernel, block) and kept, so a process that drives several devices sizes each
// grid for its own device and no launch pays for an occupancy query.
static std::mutex g_occ_mutex;
static std::map<std::tuple<int, const void *, int>, int> g_occ_grid;

cudaError_t persistent_grid(const void *kern, int block, int *grid) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const auto key = std::make_tuple(dev, kern, block);
    {
        std::lock_guard<std::mutex> lock(g_occ_mutex);
        auto it = g_occ_grid.find(key);
        if (it != g_occ_grid.end()) {
            *grid = it->second;
            return cudaSuccess;
        }
    }
    int sms = 0, occ = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, block, 0);
    if (e != cudaSuccess) return e;
    if (occ < 1) occ = 1;
    *grid = sms * occ;
    std::lock_guard<std::mutex> lock(g_occ_mutex);
    g_occ_grid[key] = *grid;
    return cudaSuccess;
}
}  // namespace joker

extern "C" uint64_t joker_launch_count(void) { return (uint64_t)joker::g_launches.load(); }

extern "C" int joker_abi_version(void) { return JOKER_ABI_VERSION; }
extern "C" const char *joker_last_error(void) { return g_err.c_str(); }

extern "C" double joker_key_to_double(uint64_t key) { return key_to_double(key); }

// ---------------------------------------------------------------- star table
static void split_ff(double v, float &hi, float &lo) {
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// Inverse and log-determinant of a small symmetric positive-definite matrix
// (Cholesky, long double).  Returns false if not positive definite.
static bool spd_inverse(int n, const long double *A, long double *Ainv, long double &logdet) {
    std::vector<long double> Lc(n * n, 0.0L);
    logdet = 0.0L;
    for (int j = 0; j < n; ++j) {
        long double d = A[j * n + j];
        for (int k = 0; k < j; ++k) d -= Lc[j * n + k] * Lc[j * n + k];
        if (!(d > 0.0L)) return false;
        const long double ljj = sqrtl(d);
        Lc[j * n + j] = ljj;
        logdet += 2.0L * logl(ljj);
        for (int i = j + 1; i < n; ++i) {
            long double v = A[i * n + j];
            for (int k = 0; k < j; ++k) v -= Lc[i * n + k] * Lc[j * n + k];
            Lc[i * n + j] = v / ljj;
        }
    }
    // inverse column by column
    std::vector<long double> col(n);
    for (int c = 0; c < n; ++c) {
        for (int i = 0; i < n; ++i) {
            long double v = (i == c) ? 1.0L : 0.0L;
            for (int k = 0; k < i; ++k) v -= Lc[i * n + k] * col[k];
            col[i] = v / Lc[i * n + i];
        }
        for (int i = n - 1; i >= 0; --i) {
            long double v = col[i];
            for (int k = i + 1; k < n; ++k) v -= Lc[k * n + i] * col[k];
            col[i] = v / Lc[i * n + i];
        }
        for (int i = 0; i < n; ++i) Ainv[i * n + c] = col[i];
    }
    return true;
}

// Per-star preparation on the host, in FP64 / long double: the StarRec
// constants and the epoch records of both kernels.  Epoch records are written
// at rec64 / rec32 (n epochs each); the record's epoch_off is set by the caller.
static int prep_star(int k, int L, int jitter_mode, int n, const double *t, const double *rv,
                     const double *ivar, double t_ref, const double *trend_M, const double *muk,
                     const double *lamk, const double *kp, StarRec &r, double *rec64,
                     float *rec32) {
    const int T = L - 1;
    const long double LOG2PI = logl(2.0L * 3.141592653589793238462643383279502884L);
    for (int i = 0; i < n; ++i)
        if (!(ivar[i] > 0.0) || !std::isfinite(ivar[i]) || !std::isfinite(t[i]) ||
            !std::isfinite(rv[i]))
            return fail(JOKER_EINVAL, "star %d epoch %d: ivar must be positive and finite, t and "
                                      "rv finite", k, i);
    if (T > 0)
        for (int i = 0; i < n; ++i)
            if (trend_M[(size_t)i * T] != 1.0)
                return fail(JOKER_EINVAL, "star %d: column 0 of trend_M must be 1 (the constant "
                                          "v0 term of the reference's design matrix)", k);
    // finite and positive: an infinite variance makes the prior's normalisation
    // (sum log lambda) infinite, where the reference's arithmetic gives NaN
    for (int j = 0; j < L; ++j)
        if (!(lamk[j] > 0.0 && std::isfinite(lamk[j])) && !(j == 0 && kp[0] != 0.0))
            return fail(JOKER_EINVAL, "star %d: prior variance lambda[%d] must be positive and "
                                      "finite", k, j);
    if (kp[0] != 0.0 && !(kp[1] > 0.0 && kp[2] > 0.0 && kp[3] > 0.0))
        return fail(JOKER_EINVAL, "star %d: scaled K prior needs sigma_K0, P0, max_K > 0", k);
    const int32_t keep_off = r.epoch_off;
    memset(&r, 0, sizeof r);
    r.epoch_off = keep_off;
    r.n_epochs = n;
    r.k_scaled = kp[0] != 0.0;
    r.mu0 = muk[0];
    r.lam0 = lamk[0];
    r.sigK0sq = kp[1] * kp[1];
    r.P0 = kp[2];
    r.maxK2 = kp[3] * kp[3];
    r.log_kscale = r.k_scaled ? std::log(r.sigK0sq) + 2.0 / 3.0 * std::log(r.P0) : 0.0;
    r.log_maxK2 = r.k_scaled ? std::log(r.maxK2) : 0.0;
    r.log_kscale_f = (float)r.log_kscale;
    r.log_maxK2_f = (float)r.log_maxK2;
    r.log_lam0_f = (float)std::log(r.lam0);
    for (int j = 0; j < L; ++j) r.lam[j] = lamk[j];
    for (int j = 0; j < L; ++j)
        r.ilam[j] = lamk[j] > 0.0 ? (double)(1.0L / (long double)lamk[j]) : 0.0;
    r.iP0 = r.k_scaled ? (double)(1.0L / (long double)r.P0) : 0.0;
    for (int j = 0; j < L; ++j) r.mu[j] = muk[j];
    std::vector<long double> C(T * T, 0.0L), c(T, 0.0L), Cinv(T * T, 0.0L);
    long double Syy = 0.0L, slog_ivar = 0.0L, slog_lam = 0.0L, sw = 0.0L;
    for (int j = 1; j < L; ++j) slog_lam += logl((long double)lamk[j]);
    for (int i = 0; i < n; ++i) {
        const double dt = t[i] - t_ref;
        long double yp = rv[i];
        for (int j = 1; j < L; ++j) yp -= (long double)muk[j] * trend_M[(size_t)i * T + (j - 1)];
        const long double w = ivar[i];
        sw += w;
        Syy += w * yp * yp;
        slog_ivar += logl(w);
        for (int j = 0; j < T; ++j) {
            const long double Tj = trend_M[(size_t)i * T + j];
            c[j] += w * Tj * yp;
            for (int m = 0; m < T; ++m) C[j * T + m] += w * Tj * trend_M[(size_t)i * T + m];
        }
        // FP64 record: dt, y', ivar, T_1..T_{L-1}
        double *r64 = rec64 + (size_t)i * REC64;
        for (int q = 0; q < REC64; ++q) r64[q] = 0.0;
        r64[0] = dt;
        r64[1] = (double)yp;
        r64[2] = ivar[i];
        for (int j = 0; j < T; ++j) r64[3 + j] = trend_M[(size_t)i * T + j];
        // mixed record
        float *r32 = rec32 + (size_t)i * REC32;
        for (int q = 0; q < REC32; ++q) r32[q] = 0.0f;
        split_ff(dt, r32[0], r32[1]);
        if (jitter_mode == JOKER_JITTER_REFERENCE) {
            // dt, w, w y', w T_j
            split_ff(ivar[i], r32[2], r32[3]);
            split_ff((double)(w * yp), r32[4], r32[5]);
            for (int j = 0; j < T; ++j)
                split_ff((double)(w * (long double)trend_M[(size_t)i * T + j]), r32[6 + 2 * j],
                         r32[7 + 2 * j]);
        } else {
            // dt, ivar, y', y'^2, T_j
            r32[2] = (float)ivar[i];
            r32[3] = 0.0f;
            split_ff((double)yp, r32[4], r32[5]);
            split_ff((double)(yp * yp), r32[6], r32[7]);
            for (int j = 0; j < T; ++j)
                split_ff(trend_M[(size_t)i * T + j], r32[8 + 2 * j], r32[9 + 2 * j]);
        }
    }
    for (int j = 0; j < T; ++j) C[j * T + j] += 1.0L / (long double)lamk[j + 1];
    long double logdetC = 0.0L;
    if (T > 0 && !spd_inverse(T, C.data(), Cinv.data(), logdetC))
        return fail(JOKER_EINVAL, "star %d: trend block of the linear system is not positive definite", k);
    long double cCc = 0.0L;
    for (int j = 0; j < T; ++j) {
        long double v = 0.0L;
        for (int m = 0; m < T; ++m) v += Cinv[j * T + m] * c[m];
        r.cC[j + 1] = (double)v;
        cCc += c[j] * v;
        for (int m = 0; m < T; ++m) r.Cinv[(j + 1) * MAXL + (m + 1)] = (double)Cinv[j * T + m];
    }
    r.chi2_0 = (double)(Syy - cCc);
    split_ff(r.chi2_0, r.chi2_0_hi, r.chi2_0_lo);
    for (int j = 1; j < L; ++j) {
        split_ff(r.cC[j], r.cC_hi[j], r.cC_lo[j]);
        for (int m = 1; m < L; ++m)
            split_ff(r.Cinv[j * MAXL + m], r.Cinv_hi[j * MAXL + m], r.Cinv_lo[j * MAXL + m]);
        split_ff((double)(1.0L / (long double)lamk[j]), r.ilam_hi[j], r.ilam_lo[j]);
    }
    r.sum_ivar = (float)(sw * (1.0L + 1e-6L));   // rounded up: an upper bound
    r.mu0_f = (float)muk[0];
    r.mu0_zero = muk[0] == 0.0;
    r.logdet_const = (double)(n * LOG2PI - slog_ivar + slog_lam + logdetC);
    r.log_norm_rest = (double)(n * LOG2PI + slog_lam);
    r.sum_log_ivar = (double)slog_ivar;
    // FP32-sum path: the residual of the trend-only fit r_c = y' - T^T beta0
    // (beta0 = C^-1 c, as stored in cC) and the magnitudes its bound needs
    long double Cn = 0.0L, ivmax = 0.0L, Wjj[MAXL] = {0.0L}, kappa = 0.0L, dtmax = 0.0L,
                swdt2 = 0.0L;
    for (int j = 1; j < L; ++j) kappa += (long double)r.cC[j] * r.cC[j] / (long double)lamk[j];
    for (int i = 0; i < n; ++i) {
        long double yp = rv[i];
        for (int j = 1; j < L; ++j) yp -= (long double)muk[j] * trend_M[(size_t)i * T + (j - 1)];
        long double rc = yp;
        for (int j = 1; j < L; ++j) rc -= (long double)r.cC[j] * trend_M[(size_t)i * T + (j - 1)];
        const long double w = ivar[i];
        Cn += w * rc * rc;
        ivmax = std::max(ivmax, w);
        for (int j = 1; j < L; ++j) {
            const long double Tj = trend_M[(size_t)i * T + (j - 1)];
            Wjj[j] += w * Tj * Tj;
        }
        const long double adt = std::fabs(t[i] - t_ref);
        dtmax = std::max(dtmax, adt);
        swdt2 += (long double)ivar[i] * adt * adt;
        float *r32 = rec32 + (size_t)i * REC32;
        // dt split for the FP32-sum kernel's phase: dth with 12 significant
        // bits (exact in a float), dtl the rest.  Words 16 and 17 are free in
        // every layout that kernel reads (with the jitter it takes L <= 3; at
        // L = 6 they hold the float-float kernel's last trend column)
        if (jitter_mode != JOKER_JITTER_APPLIED || L <= 5) {
            const double dt = t[i] - t_ref;
            int ex = 0;
            const double mant = std::frexp(dt, &ex);
            const double dth = std::ldexp(std::nearbyint(std::ldexp(mant, 12)), ex - 12);
            r32[16] = (float)dth;
            r32[17] = (float)(dt - dth);
        }
        r32[18] = (float)rc;
        r32[19] = (float)(w * rc);
    }
    // early-exit checkpoints of the fused pass (L <= 3): the partial sums'
    // constants after the first k epochs, in the epochs' record order
    r.n_ck = 0;
    if (L <= 3) {
        static const int sched[MAX_CK] = {8, 12, 16, 24, 32, 48, 64, 96};
        long double P[2] = {0.0L, 0.0L}, Ck = 0.0L, H[4] = {0.0L, 0.0L, 0.0L, 0.0L};
        int q = 0, i = 0;
        for (int c = 0; c < MAX_CK; ++c) {
            const int kend = sched[c];
            if (kend >= n) break;
            for (; i < kend; ++i) {
                long double yp = rv[i];
                for (int j = 1; j < L; ++j)
                    yp -= (long double)muk[j] * trend_M[(size_t)i * T + (j - 1)];
                long double rc = yp;
                for (int j = 1; j < L; ++j)
                    rc -= (long double)r.cC[j] * trend_M[(size_t)i * T + (j - 1)];
                const long double w = ivar[i];
                Ck += w * rc * rc;
                for (int j = 0; j < T; ++j) {
                    const long double Tj = trend_M[(size_t)i * T + j];
                    P[j] += w * rc * Tj;
                    for (int m = 0; m < T; ++m) H[j * T + m] += w * Tj * trend_M[(size_t)i * T + m];
                }
            }
            long double Hc[4], Hinv[4] = {0.0L, 0.0L, 0.0L, 0.0L}, ldH = 0.0L;
            for (int j = 0; j < T * T; ++j) Hc[j] = H[j];
            for (int j = 0; j < T; ++j) Hc[j * T + j] += 1.0L / (long double)lamk[j + 1];
            if (T > 0 && !spd_inverse(T, Hc, Hinv, ldH)) break;
            float *ck = r.ck[q];
            for (int j = 0; j < 8; ++j) ck[j] = 0.0f;
            for (int j = 0; j < T; ++j)
                ck[j] = (float)(P[j] - (long double)r.cC[j + 1] / (long double)lamk[j + 1]);
            ck[2] = (float)(Ck + kappa);
            if (T >= 1) ck[3] = (float)Hinv[0];
            if (T == 2) { ck[4] = (float)Hinv[1]; ck[5] = (float)Hinv[3]; }
            ck[6] = (float)ldH;
            r.ck_k[q] = kend;
            ++q;
        }
        r.n_ck = q;
    }
    // all epochs (L <= 4): P = 0 (T W0 r_c = Lambda_T^-1 beta0), C + kappa =
    // chi2_0, H = C (the folded trend block).  With three trend columns the
    // free P slots hold the third row of C^-1: {Hi13, Hi23, C + kappa, Hi11,
    // Hi12, Hi22, log det C, Hi33}
    for (int j = 0; j < 8; ++j) r.ck_full[j] = 0.0f;
    if (L <= 4) {
        r.ck_full[2] = (float)(Cn + kappa);
        if (T >= 1) r.ck_full[3] = (float)Cinv[0];
        if (T >= 2) { r.ck_full[4] = (float)Cinv[1]; r.ck_full[5] = (float)Cinv[T + 1]; }
        if (T == 3) {
            r.ck_full[0] = (float)Cinv[2];
            r.ck_full[1] = (float)Cinv[5];
            r.ck_full[7] = (float)Cinv[8];
        }
        r.ck_full[6] = (float)logdetC;
    }
    split_ff((double)kappa, r.kappa_hi, r.kappa_lo);
    split_ff(r.logdet_const, r.ldc_hi, r.ldc_lo);
    split_ff((double)(n * LOG2PI + slog_lam - slog_ivar), r.lnr_hi, r.lnr_lo);
    r.Cn = (float)(Cn * (1.0L + 1e-6L));
    r.ivar_max = (float)(ivmax * (1.0L + 1e-6L));
    // the split phase rounds to at most 2.5 2^-34 |dt| / P cycles; the bound
    // takes the column error through its ivar-weighted norm, so the
    // ivar-weighted RMS of |dt| stands for |dt| (the largest |dt| when the
    // weights are not finite)
    long double rms = sw > 0.0L ? sqrtl(swdt2 / sw) : dtmax;
    if (!(rms <= dtmax)) rms = dtmax;
    r.phase_c = (float)(rms * (2.0L * 3.141592653589793238462643383279502884L * 2.5L *
                               0x1p-34L * (1.0L + 1e-6L)));
    for (int j = 1; j < L; ++j) r.Wjj[j] = (float)(Wjj[j] * (1.0L + 1e-6L));
    return JOKER_OK;
}

extern "C" int joker_stars_create(joker_stars **out, int n_stars, int n_linear,
                                  const int64_t *epoch_offsets, const double *t,
                                  const double *rv, const double *ivar, const double *t_ref,
                                  const double *trend_M, const double *mu,
                                  const double *lambda, const double *k_prior,
                                  int jitter_mode) {
    if (!out) return fail(JOKER_EINVAL, "joker_stars_create: out is NULL");
    *out = nullptr;
    if (n_stars <= 0) return fail(JOKER_EINVAL, "joker_stars_create: n_stars must be > 0");
    if (n_linear < 1 || n_linear > JOKER_MAX_LINEAR)
        return fail(JOKER_EINVAL, "joker_stars_create: n_linear=%d outside [1, %d]", n_linear,
                    JOKER_MAX_LINEAR);
    if (jitter_mode != JOKER_JITTER_REFERENCE && jitter_mode != JOKER_JITTER_APPLIED)
        return fail(JOKER_EINVAL, "joker_stars_create: unknown jitter_mode %d", jitter_mode);
    if (!epoch_offsets || !t || !rv || !ivar || !t_ref || !mu || !lambda || !k_prior ||
        (n_linear > 1 && !trend_M))
        return fail(JOKER_EINVAL, "joker_stars_create: NULL array argument");
    if (epoch_offsets[0] != 0) return fail(JOKER_EINVAL, "epoch_offsets[0] must be 0");
    const int L = n_linear, T = n_linear - 1;
    int max_ep = 0;
    for (int k = 0; k < n_stars; ++k) {
        const int64_t n = epoch_offsets[k + 1] - epoch_offsets[k];
        if (n <= 0) return fail(JOKER_EINVAL, "star %d has no epochs", k);
        if (n > (int64_t)1 << 30) return fail(JOKER_ERANGE, "star %d: too many epochs", k);
        max_ep = std::max<int>(max_ep, (int)n);
    }
    const int64_t NE = epoch_offsets[n_stars];
    std::vector<StarRec> recs(n_stars);
    std::vector<double> ep64((size_t)NE * REC64, 0.0);
    std::vector<float> ep32((size_t)NE * REC32, 0.0f);
    for (int k = 0; k < n_stars; ++k) {
        const int64_t e0 = epoch_offsets[k];
        const int n = (int)(epoch_offsets[k + 1] - e0);
        recs[k].epoch_off = (int32_t)e0;
        const int rc = prep_star(k, L, jitter_mode, n, t + e0, rv + e0, ivar + e0, t_ref[k],
                                 T > 0 ? trend_M + (size_t)e0 * T : nullptr,
                                 mu + (size_t)k * L, lambda + (size_t)k * L, k_prior + (size_t)k * 4,
                                 recs[k], &ep64[(size_t)e0 * REC64], &ep32[(size_t)e0 * REC32]);
        if (rc != JOKER_OK) return rc;
    }
    std::vector<int> order(n_stars);
    for (int k = 0; k < n_stars; ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return recs[a].n_epochs > recs[b].n_epochs;
    });

    joker_stars *s = new joker_stars();
    s->n_stars = n_stars;
    s->L = L;
    s->jitter = jitter_mode;
    s->max_epochs = max_ep;
    s->total_epochs = NE;
    s->off.assign(epoch_offsets, epoch_offsets + n_stars + 1);
    auto cleanup = [&]() { joker_stars_destroy(s); };
    cudaError_t e;
    if ((e = cudaMalloc(&s->d_stars, sizeof(StarRec) * n_stars)) != cudaSuccess ||
        (e = cudaMalloc(&s->d_ep64, sizeof(double) * ep64.size())) != cudaSuccess ||
        (e = cudaMalloc(&s->d_ep32, sizeof(float) * ep32.size())) != cudaSuccess ||
        (e = cudaMalloc(&s->d_queue, sizeof(int) * 4)) != cudaSuccess ||
        (e = cudaMalloc(&s->d_order, sizeof(int) * n_stars)) != cudaSuccess) {
        cleanup();
        return fail(JOKER_ENOMEM, "joker_stars_create: cudaMalloc: %s", cudaGetErrorString(e));
    }
    if ((e = cudaMemcpy(s->d_stars, recs.data(), sizeof(StarRec) * n_stars,
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(s->d_ep64, ep64.data(), sizeof(double) * ep64.size(),
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(s->d_ep32, ep32.data(), sizeof(float) * ep32.size(),
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(s->d_order, order.data(), sizeof(int) * n_stars,
                        cudaMemcpyHostToDevice)) != cudaSuccess) {
        cleanup();
        return fail(JOKER_ECUDA, "joker_stars_create: cudaMemcpy: %s", cudaGetErrorString(e));
    }
    *out = s;
    return JOKER_OK;
}

// A table of n_slots empty stars with room for max_epochs epochs each; slots
// are filled (and refilled) by joker_stars_set.
extern "C" int joker_stars_create_slots(joker_stars **out, int n_slots, int max_epochs,
                                        int n_linear, int jitter_mode) {
    if (!out) return fail(JOKER_EINVAL, "joker_stars_create_slots: out is NULL");
    *out = nullptr;
    if (n_slots <= 0 || max_epochs <= 0)
        return fail(JOKER_EINVAL, "joker_stars_create_slots: n_slots and max_epochs must be > 0");
    if ((int64_t)n_slots * max_epochs > ((int64_t)1 << 31) - 1)
        return fail(JOKER_ERANGE, "joker_stars_create_slots: n_slots * max_epochs too large");
    if (n_linear < 1 || n_linear > JOKER_MAX_LINEAR)
        return fail(JOKER_EINVAL, "joker_stars_create_slots: n_linear=%d outside [1, %d]",
                    n_linear, JOKER_MAX_LINEAR);
    if (jitter_mode != JOKER_JITTER_REFERENCE && jitter_mode != JOKER_JITTER_APPLIED)
        return fail(JOKER_EINVAL, "joker_stars_create_slots: unknown jitter_mode %d", jitter_mode);
    joker_stars *s = new joker_stars();
    s->n_stars = n_slots;
    s->L = n_linear;
    s->jitter = jitter_mode;
    s->max_epochs = max_epochs;
    s->slot_epochs = max_epochs;
    s->total_epochs = (int64_t)n_slots * max_epochs;
    s->off.resize(n_slots + 1);
    for (int k = 0; k <= n_slots; ++k) s->off[k] = (int64_t)k * max_epochs;
    std::vector<StarRec> recs(n_slots);
    memset(recs.data(), 0, sizeof(StarRec) * n_slots);
    for (int k = 0; k < n_slots; ++k) recs[k].epoch_off = (int32_t)(k * max_epochs);
    std::vector<int> order(n_slots);
    for (int k = 0; k < n_slots; ++k) order[k] = k;
    cudaError_t e;
    if ((e = cudaMalloc(&s->d_stars, sizeof(StarRec) * n_slots)) != cudaSuccess ||
        (e = cudaMalloc(&s->d_ep64, sizeof(double) * REC64 * s->total_epochs)) != cudaSuccess ||
        (e = cudaMalloc(&s->d_ep32, sizeof(float) * REC32 * s->total_epochs)) != cudaSuccess ||
        (e = cudaMalloc(&s->d_queue, sizeof(int) * 4)) != cudaSuccess ||
        (e = cudaMalloc(&s->d_order, sizeof(int) * n_slots)) != cudaSuccess ||
        (e = cudaMemcpy(s->d_stars, recs.data(), sizeof(StarRec) * n_slots,
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(s->d_order, order.data(), sizeof(int) * n_slots,
                        cudaMemcpyHostToDevice)) != cudaSuccess) {
        joker_stars_destroy(s);
        return fail(JOKER_ENOMEM, "joker_stars_create_slots: %s", cudaGetErrorString(e));
    }
    *out = s;
    return JOKER_OK;
}

// Fill slot `slot` of a slot table with one star (the per-star arguments of
// joker_stars_create).  The copies are ordered on `stream`; the host arrays
// are read before the call returns.
extern "C" int joker_stars_set(joker_stars *s, int slot, int n_epochs, const double *t,
                               const double *rv, const double *ivar, double t_ref,
                               const double *trend_M, const double *mu, const double *lambda,
                               const double *k_prior, void *stream) {
    if (!s) return fail(JOKER_EINVAL, "joker_stars_set: NULL handle");
    if (s->slot_epochs <= 0) return fail(JOKER_EINVAL, "joker_stars_set: not a slot table");
    if (slot < 0 || slot >= s->n_stars)
        return fail(JOKER_EINVAL, "joker_stars_set: slot %d outside [0, %d)", slot, s->n_stars);
    if (n_epochs <= 0 || n_epochs > s->slot_epochs)
        return fail(JOKER_ERANGE, "joker_stars_set: %d epochs outside [1, %d]", n_epochs,
                    s->slot_epochs);
    if (!t || !rv || !ivar || !mu || !lambda || !k_prior || (s->L > 1 && !trend_M))
        return fail(JOKER_EINVAL, "joker_stars_set: NULL array argument");
    StarRec r;
    memset(&r, 0, sizeof r);
    r.epoch_off = slot * s->slot_epochs;
    std::vector<double> r64((size_t)n_epochs * REC64);
    std::vector<float> r32((size_t)n_epochs * REC32);
    const int rc = prep_star(slot, s->L, s->jitter, n_epochs, t, rv, ivar, t_ref, trend_M, mu,
                             lambda, k_prior, r, r64.data(), r32.data());
    if (rc != JOKER_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(cudaMemcpyAsync(s->d_ep64 + (size_t)r.epoch_off * REC64, r64.data(),
                             sizeof(double) * r64.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->d_ep32 + (size_t)r.epoch_off * REC32, r32.data(),
                             sizeof(float) * r32.size(), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(s->d_stars + slot, &r, sizeof(StarRec), cudaMemcpyHostToDevice, st));
    // pageable sources: staged before the calls return
    return JOKER_OK;
}

extern "C" int joker_stars_destroy(joker_stars *s) {
    if (!s) return JOKER_OK;
    cudaFree(s->d_stars);
    cudaFree(s->d_ep64);
    cudaFree(s->d_ep32);
    cudaFree(s->d_queue);
    cudaFree(s->d_order);
    delete s;
    return JOKER_OK;
}

extern "C" int joker_stars_info(const joker_stars *s, int *n_stars, int *n_linear,
                                int64_t *total_epochs, int *max_epochs) {
    if (!s) return fail(JOKER_EINVAL, "joker_stars_info: NULL handle");
    if (n_stars) *n_stars = s->n_stars;
    if (n_linear) *n_linear = s->L;
    if (total_epochs) *total_epochs = s->total_epochs;
    if (max_epochs) *max_epochs = s->max_epochs;
    return JOKER_OK;
}

// ---------------------------------------------------------------- prior cache
extern "C" int joker_cache_create(joker_cache **out, int64_t capacity) {
    if (!out) return fail(JOKER_EINVAL, "joker_cache_create: out is NULL");
    *out = nullptr;
    if (capacity <= 0) return fail(JOKER_EINVAL, "joker_cache_create: capacity must be > 0");
    joker_cache *c = new joker_cache();
    c->cap = capacity;
    cudaError_t e;
    const size_t n = (size_t)capacity;
    if ((e = cudaMalloc(&c->P, 8 * n)) != cudaSuccess || (e = cudaMalloc(&c->E, 8 * n)) != cudaSuccess ||
        (e = cudaMalloc(&c->OM, 8 * n)) != cudaSuccess || (e = cudaMalloc(&c->M0, 8 * n)) != cudaSuccess ||
        (e = cudaMalloc(&c->S, 8 * n)) != cudaSuccess ||
        (e = cudaMalloc(&c->mx_a, 16 * n)) != cudaSuccess ||
        (e = cudaMalloc(&c->mx_b, 16 * n)) != cudaSuccess ||
        (e = cudaMalloc(&c->mx_s2, 4 * n)) != cudaSuccess ||
        (e = cudaMalloc(&c->flag, sizeof(int))) != cudaSuccess) {
        joker_cache_destroy(c);
        return fail(JOKER_ENOMEM, "joker_cache_create(%lld): %s", (long long)capacity,
                    cudaGetErrorString(e));
    }
    *out = c;
    return JOKER_OK;
}

extern "C" int joker_cache_destroy(joker_cache *c) {
    if (!c) return JOKER_OK;
    if (!c->view) {
        cudaFree(c->P); cudaFree(c->E); cudaFree(c->OM); cudaFree(c->M0); cudaFree(c->S);
    }
    cudaFree(c->mx_a); cudaFree(c->mx_b); cudaFree(c->mx_s2); cudaFree(c->flag);
    delete c;
    return JOKER_OK;
}

extern "C" int64_t joker_cache_capacity(const joker_cache *c) { return c ? c->cap : -1; }

namespace joker {
cudaError_t launch_prior_sample(const joker_prior_spec &spec, uint64_t seed, int64_t first_index,
                                int64_t n, int64_t row0, double *P, double *E, double *OM,
                                double *M0, double *S, float4 *mx_a, float4 *mx_b, float *mx_s2,
                                double *packed, int *bad, cudaStream_t st);
}  // namespace joker

// Prior samples drawn on the device into cache rows [row0, row0 + n).  Waits
// for the stream to read the status word.
extern "C" int joker_prior_sample(joker_cache *c, int64_t row0, int64_t n,
                                  const joker_prior_spec *spec, uint64_t seed,
                                  int64_t first_index, double *d_packed, void *stream) {
    if (!c || !spec) return fail(JOKER_EINVAL, "joker_prior_sample: NULL argument");
    if (c->view) return fail(JOKER_EINVAL, "joker_prior_sample: a cache view holds no storage");
    if (n < 0 || row0 < 0 || row0 + n > c->cap || first_index < 0)
        return fail(JOKER_ERANGE, "joker_prior_sample: rows [%lld, %lld) outside the cache (%lld)",
                    (long long)row0, (long long)(row0 + n), (long long)c->cap);
    if (!(spec->P_min > 0.0 && spec->P_max > spec->P_min && std::isfinite(spec->P_max)))
        return fail(JOKER_EINVAL, "joker_prior_sample: need 0 < P_min < P_max");
    if (!(spec->e_alpha > 0.0 && spec->e_beta > 0.0 && std::isfinite(spec->e_alpha) &&
          std::isfinite(spec->e_beta)))
        return fail(JOKER_EINVAL, "joker_prior_sample: Beta shapes must be > 0");
    if (spec->s_kind == JOKER_S_FIXED) {
        if (!std::isfinite(spec->s_value) || spec->s_value < 0.0)
            return fail(JOKER_EINVAL, "joker_prior_sample: fixed s must be finite and >= 0");
    } else if (spec->s_kind == JOKER_S_LOGNORMAL) {
        if (!std::isfinite(spec->s_mu) || !(spec->s_sigma >= 0.0) || !std::isfinite(spec->s_sigma))
            return fail(JOKER_EINVAL, "joker_prior_sample: bad log-normal s parameters");
    } else {
        return fail(JOKER_EINVAL, "joker_prior_sample: unknown s_kind %d", spec->s_kind);
    }
    if (n == 0) return JOKER_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int bad = 0;
    CUDA_TRY(cudaMemsetAsync(c->flag, 0, sizeof(int), st));
    CUDA_TRY(launch_prior_sample(*spec, seed, first_index, n, row0, c->P, c->E, c->OM, c->M0, c->S,
                                 c->mx_a, c->mx_b, c->mx_s2, d_packed, c->flag, st));
    CUDA_TRY(cudaMemcpyAsync(&bad, c->flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (bad) return fail(JOKER_ERANGE, "joker_prior_sample: %d samples hit the gamma retry limit", bad);
    return JOKER_OK;
}

// A cache over the caller's packed (n, 5) FP64 chunk, without a copy: the
// FP64 columns alias it (stride 5) and the mixed kernel prepares each sample
// in registers.  The chunk may be device memory, or pinned host memory that
// the device reads through its mapped address (every ln L call then streams
// 40 bytes per sample over the host link).  Pageable host memory is taken
// only where the device can address it (cudaDevAttrPageableMemoryAccess).
// The device address through which a kernel reads caller memory p: p itself
// for device or managed memory and on systems with pageable-memory access, the
// mapped address for pinned host memory.
static int device_view_ptr(const double *p, const double **dptr, const char *who) {
    if (((uintptr_t)p) % 8) return fail(JOKER_EINVAL, "%s: pointer not 8-byte aligned", who);
    cudaPointerAttributes at;
    CUDA_TRY(cudaPointerGetAttributes(&at, p));
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
        *dptr = p;
    } else if (at.type == cudaMemoryTypeHost) {
        void *d = nullptr;
        CUDA_TRY(cudaHostGetDevicePointer(&d, const_cast<double *>(p), 0));
        *dptr = (const double *)d;
    } else {
        int dev = 0, pageable = 0;
        CUDA_TRY(cudaGetDevice(&dev));
        CUDA_TRY(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev));
        if (!pageable)
            return fail(JOKER_EINVAL, "%s: host memory must be pinned (cudaHostAlloc / "
                                      "cudaHostRegister) on this system", who);
        *dptr = p;
    }
    return JOKER_OK;
}

extern "C" int joker_cache_create_view(joker_cache **out, const double *chunk, int64_t n) {
    if (!out) return fail(JOKER_EINVAL, "joker_cache_create_view: out is NULL");
    *out = nullptr;
    if (!chunk || n <= 0) return fail(JOKER_EINVAL, "joker_cache_create_view: empty chunk");
    const double *dptr = nullptr;
    const int rc = device_view_ptr(chunk, &dptr, "joker_cache_create_view");
    if (rc != JOKER_OK) return rc;
    joker_cache *c = new joker_cache();
    c->cap = n;
    c->view = true;
    c->stride = 5;
    c->P = const_cast<double *>(dptr);
    c->E = c->P + 1; c->OM = c->P + 2; c->M0 = c->P + 3; c->S = c->P + 4;
    *out = c;
    return JOKER_OK;
}

extern "C" int joker_cache_bind(joker_cache **out, const double *P, const double *e,
                                const double *omega, const double *M0, const double *s,
                                int64_t n) {
    if (!out) return fail(JOKER_EINVAL, "joker_cache_bind: out is NULL");
    *out = nullptr;
    if (n <= 0) return fail(JOKER_EINVAL, "joker_cache_bind: n must be > 0");
    if (!P || !e || !omega || !M0 || !s) return fail(JOKER_EINVAL, "joker_cache_bind: NULL column");
    const double *cols[5] = {P, e, omega, M0, s};
    const double *d[5];
    for (int k = 0; k < 5; ++k) {
        const int rc = device_view_ptr(cols[k], &d[k], "joker_cache_bind");
        if (rc != JOKER_OK) return rc;
    }
    joker_cache *c = new joker_cache();
    c->cap = n;
    c->view = true;
    c->stride = 1;
    c->P = const_cast<double *>(d[0]);
    c->E = const_cast<double *>(d[1]);
    c->OM = const_cast<double *>(d[2]);
    c->M0 = const_cast<double *>(d[3]);
    c->S = const_cast<double *>(d[4]);
    *out = c;
    return JOKER_OK;
}

extern "C" int joker_cache_load(joker_cache *c, const double *d_chunk, int64_t n, int64_t row0,
                                void *stream) {
    if (!c || (!d_chunk && n > 0)) return fail(JOKER_EINVAL, "joker_cache_load: NULL argument");
    if (c->view) return fail(JOKER_EINVAL, "joker_cache_load: a cache view holds no storage");
    if (n < 0 || row0 < 0 || row0 + n > c->cap)
        return fail(JOKER_ERANGE, "joker_cache_load: rows [%lld, %lld) exceed capacity %lld",
                    (long long)row0, (long long)(row0 + n), (long long)c->cap);
    CUDA_TRY(launch_prepare(d_chunk, n, row0, c->P, c->E, c->OM, c->M0, c->S, c->mx_a, c->mx_b,
                            c->mx_s2, (cudaStream_t)stream));
    return JOKER_OK;
}

// ---------------------------------------------------------------- likelihood
static int run_lnl(const joker_stars *s, int precision, LnlArgs a, int block,
                   cudaStream_t st) {
    CUDA_TRY(cudaMemsetAsync(s->d_queue, 0, sizeof(int), st));
    CUDA_TRY(launch_lnl(precision, s->L, s->jitter == JOKER_JITTER_APPLIED, a, block, st));
    return JOKER_OK;
}
extern "C" int joker_batch_marginal_ln_likelihood(const joker_stars *s, int star,
                                                  const double *d_chunk, int64_t n_samples,
                                                  double *d_lnl, void *stream) {
    if (!s) return fail(JOKER_EINVAL, "joker_batch_marginal_ln_likelihood: NULL handle");
    if (star < 0 || star >= s->n_stars)
        return fail(JOKER_EINVAL, "star %d outside [0, %d)", star, s->n_stars);
    if (n_samples < 0) return fail(JOKER_EINVAL, "n_samples must be >= 0");
    if (n_samples == 0) return JOKER_OK;
    if (!d_chunk || !d_lnl) return fail(JOKER_EINVAL, "NULL device pointer");
    LnlArgs a;
    memset(&a, 0, sizeof a);
    a.stars = s->d_stars;
    a.ep64 = s->d_ep64;
    a.ep32 = s->d_ep32;
    a.P = d_chunk; a.e = d_chunk + 1; a.om = d_chunk + 2; a.M0 = d_chunk + 3; a.s = d_chunk + 4;
    a.stride = 5;
    a.queue = s->d_queue;
    a.lnl = d_lnl;
    a.star0 = star;
    a.n_sel = 1;
    a.row0 = 0;
    a.count = n_samples;
    a.ld = n_samples;
    a.chunk = 1024;
    a.ips = (n_samples + a.chunk - 1) / a.chunk;
    a.n_items = (int)std::min<int64_t>(a.ips, INT32_MAX);
    if (a.ips > INT32_MAX) return fail(JOKER_ERANGE, "n_samples too large for one call");
    return run_lnl(s, JOKER_FP64, a, 128, (cudaStream_t)stream);
}

static float err_c0();

namespace joker {
float mixed_err_c0() { return err_c0(); }

void stars_internals(const joker_stars *s, const StarRec **recs, const double **ep64,
                     const float **ep32, int *n_stars, int *L, int *jit, int **queue) {
    *recs = s->d_stars;
    *ep64 = s->d_ep64;
    *ep32 = s->d_ep32;
    *n_stars = s->n_stars;
    *L = s->L;
    *jit = s->jitter == JOKER_JITTER_APPLIED;
    *queue = s->d_queue;
}

void cache_internals(const joker_cache *c, int64_t *cap, const double **P, const double **E,
                     const double **OM, const double **M0, const double **S, int64_t *stride,
                     const float4 **mx_a, const float4 **mx_b, const float **mx_s2) {
    *cap = c->cap;
    *P = c->P; *E = c->E; *OM = c->OM; *M0 = c->M0; *S = c->S;
    *stride = c->stride;
    *mx_a = c->mx_a; *mx_b = c->mx_b; *mx_s2 = c->mx_s2;
}
}  // namespace joker

static float err_c0() {
    // column-error constant of the mixed kernel's bound (see joker_lnl.cu);
    // JOKER_ERR_C0 in the environment overrides it for calibration runs
    static float c0 = -1.0f;
    if (c0 < 0.0f) {
        const char *v = getenv("JOKER_ERR_C0");
        c0 = v ? (float)atof(v) : 2.0e-6f;
    }
    return c0;
}

// Arguments of an implicit-item launch over stars [star0, star0 + n_sel) x
// cache rows [row0, row0 + count) (validated by the caller); false when the
// work items do not fit in an int.
static bool lnl_args(const joker_stars *s, const joker_cache *c, int star0, int n_sel,
                     int64_t row0, int64_t count, double *d_lnl, int64_t ld,
                     uint64_t *d_max_key, int64_t chunk, LnlArgs &a) {
    memset(&a, 0, sizeof a);
    a.stars = s->d_stars;
    a.ep64 = s->d_ep64;
    a.ep32 = s->d_ep32;
    a.P = c->P; a.e = c->E; a.om = c->OM; a.M0 = c->M0; a.s = c->S;
    a.stride = c->stride;
    a.mx_a = c->mx_a; a.mx_b = c->mx_b; a.mx_s2 = c->mx_s2;
    a.queue = s->d_queue;
    a.lnl = d_lnl;
    a.max_key = (unsigned long long *)d_max_key;
    a.star0 = star0;
    a.n_sel = n_sel;
    a.row0 = row0;
    a.count = count;
    a.ld = ld;
    a.chunk = (int)chunk;
    a.ips = (count + chunk - 1) / chunk;
    a.order = (star0 == 0 && n_sel == s->n_stars) ? s->d_order : nullptr;
    const int64_t items = a.ips * n_sel;
    if (items > INT32_MAX) return false;
    a.n_items = (int)items;
    return true;
}

extern "C" int joker_lnl(const joker_stars *s, const joker_cache *c, int star0, int n_sel,
                         int64_t row0, int64_t count, int precision, double *d_lnl, int64_t ld,
                         uint64_t *d_max_key, float *d_err, uint64_t *d_bound_key, int block,
                         int64_t chunk, void *stream) {
    if (!s || !c) return fail(JOKER_EINVAL, "joker_lnl: NULL handle");
    if (precision != JOKER_FP64 && precision != JOKER_MIXED && precision != JOKER_MIXED_ACCURATE &&
        precision != JOKER_MIXED_FP64_TAIL && precision != JOKER_MIXED_FAST)
        return fail(JOKER_EINVAL, "joker_lnl: unknown precision %d", precision);
    if (star0 < 0 || n_sel < 0 || star0 + n_sel > s->n_stars)
        return fail(JOKER_EINVAL, "joker_lnl: stars [%d, %d) outside [0, %d)", star0,
                    star0 + n_sel, s->n_stars);
    if (row0 < 0 || count < 0 || row0 + count > c->cap)
        return fail(JOKER_ERANGE, "joker_lnl: rows [%lld, %lld) outside the cache (%lld)",
                    (long long)row0, (long long)(row0 + count), (long long)c->cap);
    if (n_sel == 0 || count == 0) return JOKER_OK;
    if (!d_lnl) return fail(JOKER_EINVAL, "joker_lnl: d_lnl is NULL");
    if (ld < count) return fail(JOKER_EINVAL, "joker_lnl: ld < count");
    if (block == 0) block = 128;
    if (block != 128) return fail(JOKER_EINVAL, "joker_lnl: block must be 128");
    if (chunk <= 0) chunk = 1024;
    if (chunk % block) return fail(JOKER_EINVAL, "joker_lnl: chunk must be a multiple of block");
    LnlArgs a;
    if (!lnl_args(s, c, star0, n_sel, row0, count, d_lnl, ld, d_max_key, chunk, a))
        return fail(JOKER_ERANGE, "joker_lnl: too many work items; use a larger chunk");
    if (precision != JOKER_FP64) {
        a.err = d_err;
        a.bound_key = (unsigned long long *)d_bound_key;
        a.err_c0 = err_c0();
    }
    return run_lnl(s, precision, a, block, (cudaStream_t)stream);
}

namespace joker {
cudaError_t launch_lnl_fused(int L, bool jit, const LnlArgs &a, int block, cudaStream_t st);
cudaError_t launch_accept_fused(const AcceptArgs &a, int64_t total_blocks, cudaStream_t st);
}

extern "C" int joker_lnl_fused(const joker_stars *s, const joker_cache *c, int star0, int n_sel,
                               int64_t row0, int64_t count, const uint64_t *d_pcg, int64_t first,
                               double *d_lnl, int64_t ld, uint64_t *d_max_key, float *d_err,
                               uint64_t *d_bound_key, uint32_t *d_cand, int64_t cand_ld,
                               int64_t chunk, int early_exit, void *stream) {
    if (!s || !c) return fail(JOKER_EINVAL, "joker_lnl_fused: NULL handle");
    if (star0 < 0 || n_sel < 0 || star0 + n_sel > s->n_stars)
        return fail(JOKER_EINVAL, "joker_lnl_fused: stars [%d, %d) outside [0, %d)", star0,
                    star0 + n_sel, s->n_stars);
    if (row0 < 0 || count < 0 || row0 + count > c->cap)
        return fail(JOKER_ERANGE, "joker_lnl_fused: rows [%lld, %lld) outside the cache (%lld)",
                    (long long)row0, (long long)(row0 + count), (long long)c->cap);
    if (n_sel == 0 || count == 0) return JOKER_OK;
    if (!d_lnl || !d_err || !d_bound_key || !d_pcg || !d_cand)
        return fail(JOKER_EINVAL, "joker_lnl_fused: NULL device pointer");
    if (s->jitter == JOKER_JITTER_APPLIED && s->L > 3)
        return fail(JOKER_EINVAL, "joker_lnl_fused: at most 3 linear parameters with the jitter "
                                  "applied (this table has %d)", s->L);
    if (ld < count) return fail(JOKER_EINVAL, "joker_lnl_fused: ld < count");
    if (first < 0 || first % 32)
        return fail(JOKER_EINVAL, "joker_lnl_fused: first must be a non-negative multiple of 32");
    if (cand_ld < (first + count + 31) / 32)
        return fail(JOKER_EINVAL, "joker_lnl_fused: cand_ld %lld < %lld words",
                    (long long)cand_ld, (long long)((first + count + 31) / 32));
    if (chunk <= 0) chunk = 1024;
    if (chunk % 128 || chunk > FUSED_MAX_CHUNK)
        return fail(JOKER_EINVAL, "joker_lnl_fused: chunk must be a multiple of 128 and at most %d",
                    FUSED_MAX_CHUNK);
    LnlArgs a;
    if (!lnl_args(s, c, star0, n_sel, row0, count, d_lnl, ld, d_max_key, chunk, a))
        return fail(JOKER_ERANGE, "joker_lnl_fused: too many work items; use a larger chunk");
    a.err = d_err;
    a.bound_key = (unsigned long long *)d_bound_key;
    a.err_c0 = err_c0();
    a.fa_pcg = (const unsigned long long *)d_pcg;
    a.fa_first = first;
    a.cand_words = d_cand;
    a.cand_ld = cand_ld;
    a.fa_exit = early_exit != 0 && s->L <= 3;
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(cudaMemsetAsync(s->d_queue, 0, sizeof(int), st));
    CUDA_TRY(launch_lnl_fused(s->L, s->jitter == JOKER_JITTER_APPLIED, a, 128, st));
    return JOKER_OK;
}

// ---------------------------------------------------------------- acceptance


static int64_t align256(int64_t x) { return (x + 255) & ~(int64_t)255; }

// Entries of the refinement's flag list: 64 per 8192-sample block plus 2^16;
// flagged samples beyond it are still refined, through the slower word scan.
static int64_t flag_capacity(int64_t n_blocks) { return 65536 + 64 * n_blocks; }

extern "C" int64_t joker_accept_workspace(const joker_accept_seg *segs, int n_segs) {
    if (!segs || n_segs <= 0) return 0;
    const int64_t nb = accept_blocks(segs, n_segs, nullptr);
    // the second word array and the flag list (with its two counters) serve
    // the refinement of joker_accept_refined
    return align256(sizeof(joker_accept_seg) * (int64_t)n_segs) +
           align256(8 * (int64_t)(n_segs + 1)) + align256(8 * nb) + 2 * align256(4 * 256 * nb) +
           align256(16) + align256(8 * flag_capacity(nb));
}

extern "C" int joker_accept(const joker_accept_seg *segs, int n_segs, const double *d_lnl,
                            const uint64_t *d_max_key, int u_source, const double *d_u,
                            int64_t *d_out_idx, double *d_out_lnl, int64_t *d_count,
                            void *d_work, int64_t work_bytes, void *stream) {
    if (n_segs <= 0) return JOKER_OK;
    if (!segs || !d_lnl || !d_max_key || !d_out_idx || !d_count || !d_work)
        return fail(JOKER_EINVAL, "joker_accept: NULL argument");
    if (u_source != JOKER_U_ARRAY && u_source != JOKER_U_PCG64)
        return fail(JOKER_EINVAL, "joker_accept: unknown u_source %d", u_source);
    if (u_source == JOKER_U_ARRAY && !d_u) return fail(JOKER_EINVAL, "joker_accept: d_u is NULL");
    for (int i = 0; i < n_segs; ++i)
        if (segs[i].n < 0 || segs[i].max_out < 0 || segs[i].lnl_off < 0 || segs[i].max_slot < 0)
            return fail(JOKER_EINVAL, "joker_accept: segment %d has a negative field", i);
    const int64_t need = joker_accept_workspace(segs, n_segs);
    if (work_bytes < need)
        return fail(JOKER_EINVAL, "joker_accept: workspace %lld < %lld bytes", (long long)work_bytes,
                    (long long)need);
    std::vector<int64_t> base(n_segs + 1);
    const int64_t nb = accept_blocks(segs, n_segs, base.data());
    if (nb > 0x7fffffffLL) return fail(JOKER_ERANGE, "joker_accept: too many samples in one call");
    char *w = (char *)d_work;
    joker_accept_seg *d_segs = (joker_accept_seg *)w;
    w += align256(sizeof(joker_accept_seg) * (int64_t)n_segs);
    int64_t *d_base = (int64_t *)w;
    w += align256(8 * (int64_t)(n_segs + 1));
    int64_t *d_blk = (int64_t *)w;
    w += align256(8 * nb);
    uint32_t *d_words = (uint32_t *)w;
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(cudaMemcpyAsync(d_segs, segs, sizeof(joker_accept_seg) * n_segs, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_base, base.data(), 8 * (n_segs + 1), cudaMemcpyHostToDevice, st));
    AcceptArgs a;
    memset(&a, 0, sizeof a);      // no refinement: err, exact_key, ... stay NULL
    a.segs = d_segs;
    a.blk_base = d_base;
    a.n_segs = n_segs;
    a.lnl = d_lnl;
    a.max_key = (const unsigned long long *)d_max_key;
    a.u_source = u_source;
    a.u = d_u;
    a.words = d_words;
    a.blk_count = d_blk;
    a.out_idx = d_out_idx;
    a.out_lnl = d_out_lnl;
    a.count = d_count;
    // pageable host sources are staged before cudaMemcpyAsync returns
    CUDA_TRY(launch_accept(a, nb, st));
    return JOKER_OK;
}

// Shared set-up of the refined acceptance entry points: validation, the
// segment table copied into the workspace, and the arguments.
static int refined_setup(const joker_stars *s, const joker_cache *c, const joker_accept_seg *segs,
                         int n_segs, const double *d_lnl, const float *d_err,
                         const uint64_t *d_bound_key, uint64_t *d_exact_key, int n_slots,
                         uint64_t *d_n_refined, void *d_work, int64_t work_bytes,
                         cudaStream_t st, AcceptArgs &a, int64_t &nb, const char *who) {
    if (!s || !c) return fail(JOKER_EINVAL, "%s: NULL handle", who);
    if (!segs || !d_lnl || !d_err || !d_bound_key || !d_exact_key || !d_work)
        return fail(JOKER_EINVAL, "%s: NULL argument", who);
    for (int i = 0; i < n_segs; ++i) {
        const joker_accept_seg &g = segs[i];
        if (g.n < 0 || g.max_out < 0 || g.lnl_off < 0 || g.max_slot < 0 || g.max_slot >= n_slots)
            return fail(JOKER_EINVAL, "%s: segment %d has a bad field", who, i);
        if (g.star < 0 || g.star >= s->n_stars || g.row0 < 0 || g.row0 + g.n > c->cap)
            return fail(JOKER_EINVAL, "%s: segment %d outside the stars or cache", who, i);
    }
    const int64_t need = joker_accept_workspace(segs, n_segs);
    if (work_bytes < need)
        return fail(JOKER_EINVAL, "%s: workspace %lld < %lld bytes", who, (long long)work_bytes,
                    (long long)need);
    std::vector<int64_t> base(n_segs + 1);
    nb = accept_blocks(segs, n_segs, base.data());
    if (nb > 0x7fffffffLL) return fail(JOKER_ERANGE, "%s: too many samples", who);
    char *w = (char *)d_work;
    joker_accept_seg *d_segs = (joker_accept_seg *)w;
    w += align256(sizeof(joker_accept_seg) * (int64_t)n_segs);
    int64_t *d_base = (int64_t *)w;
    w += align256(8 * (int64_t)(n_segs + 1));
    int64_t *d_blk = (int64_t *)w;
    w += align256(8 * nb);
    uint32_t *d_words = (uint32_t *)w;
    w += align256(4 * 256 * nb);
    uint32_t *d_amb = (uint32_t *)w;
    w += align256(4 * 256 * nb);
    unsigned long long *d_fcount = (unsigned long long *)w;
    w += align256(16);
    int64_t *d_flags = (int64_t *)w;
    CUDA_TRY(cudaMemcpyAsync(d_segs, segs, sizeof(joker_accept_seg) * n_segs, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(d_base, base.data(), 8 * (n_segs + 1), cudaMemcpyHostToDevice, st));
    memset(&a, 0, sizeof a);
    a.err = d_err;
    a.bound_key = (const unsigned long long *)d_bound_key;
    a.exact_key = (unsigned long long *)d_exact_key;
    a.stars = s->d_stars;
    a.ep64 = s->d_ep64;
    a.ep32 = s->d_ep32;
    a.err_c0 = err_c0();
    a.P = c->P; a.E = c->E; a.OM = c->OM; a.M0 = c->M0; a.S = c->S;
    a.stride = c->stride;
    a.L = s->L;
    a.jit = s->jitter == JOKER_JITTER_APPLIED;
    a.n_refined = (unsigned long long *)d_n_refined;
    a.amb_words = d_amb;
    a.flag_list = d_flags;
    a.flag_count = d_fcount;
    a.flag_cap = flag_capacity(nb);
    a.segs = d_segs;
    a.blk_base = d_base;
    a.n_segs = n_segs;
    a.lnl = d_lnl;
    a.max_key = (const unsigned long long *)d_exact_key;
    a.words = d_words;
    a.blk_count = d_blk;
    return JOKER_OK;
}

extern "C" int joker_refine_max(const joker_stars *s, const joker_cache *c,
                                const joker_accept_seg *segs, int n_segs, const double *d_lnl,
                                const float *d_err, const uint64_t *d_bound_key,
                                uint64_t *d_exact_key, uint64_t *d_n_refined, void *d_work,
                                int64_t work_bytes, void *stream) {
    if (n_segs <= 0) return JOKER_OK;
    int n_slots = 0;
    if (segs)
        for (int i = 0; i < n_segs; ++i) n_slots = std::max(n_slots, segs[i].max_slot + 1);
    AcceptArgs a;
    int64_t nb = 0;
    cudaStream_t st = (cudaStream_t)stream;
    const int rc = refined_setup(s, c, segs, n_segs, d_lnl, d_err, d_bound_key, d_exact_key,
                                 n_slots, d_n_refined, d_work, work_bytes, st, a, nb,
                                 "joker_refine_max");
    if (rc != JOKER_OK) return rc;
    CUDA_TRY(launch_refine_max(a, nb, st));
    return JOKER_OK;
}

extern "C" int joker_refine_band(const joker_stars *s, const joker_cache *c,
                                 const joker_accept_seg *segs, int n_segs, double *d_lnl,
                                 float *d_err, const uint64_t *d_exact_key, double band,
                                 double tol, uint64_t *d_n_refined, void *d_work,
                                 int64_t work_bytes, void *stream) {
    if (n_segs <= 0) return JOKER_OK;
    if (!(band >= 0.0) || !(tol >= 0.0))
        return fail(JOKER_EINVAL, "joker_refine_band: band and tol must be >= 0");
    int n_slots = 0;
    if (segs)
        for (int i = 0; i < n_segs; ++i) n_slots = std::max(n_slots, segs[i].max_slot + 1);
    AcceptArgs a;
    int64_t nb = 0;
    cudaStream_t st = (cudaStream_t)stream;
    // the bound maxima are not read here; the FP64 maxima stand in for them
    const int rc = refined_setup(s, c, segs, n_segs, d_lnl, d_err, d_exact_key,
                                 const_cast<uint64_t *>(d_exact_key), n_slots, d_n_refined,
                                 d_work, work_bytes, st, a, nb, "joker_refine_band");
    if (rc != JOKER_OK) return rc;
    CUDA_TRY(launch_refine_band(a, nb, band, (float)tol, st));
    return JOKER_OK;
}

extern "C" int joker_accept_refined(const joker_stars *s, const joker_cache *c,
                                    const joker_accept_seg *segs, int n_segs, double *d_lnl,
                                    float *d_err, const uint64_t *d_bound_key,
                                    uint64_t *d_exact_key, int n_slots, int max_given,
                                    int u_source, const double *d_u, int64_t *d_out_idx,
                                    double *d_out_lnl, int64_t *d_count, uint64_t *d_n_refined,
                                    void *d_work, int64_t work_bytes, void *stream) {
    if (n_segs <= 0) return JOKER_OK;
    if (!d_out_idx || !d_count) return fail(JOKER_EINVAL, "joker_accept_refined: NULL output");
    if (u_source != JOKER_U_ARRAY && u_source != JOKER_U_PCG64)
        return fail(JOKER_EINVAL, "joker_accept_refined: unknown u_source %d", u_source);
    if (u_source == JOKER_U_ARRAY && !d_u)
        return fail(JOKER_EINVAL, "joker_accept_refined: d_u is NULL");
    AcceptArgs a;
    int64_t nb = 0;
    cudaStream_t st = (cudaStream_t)stream;
    const int rc = refined_setup(s, c, segs, n_segs, d_lnl, d_err, d_bound_key, d_exact_key,
                                 n_slots, d_n_refined, d_work, work_bytes, st, a, nb,
                                 "joker_accept_refined");
    if (rc != JOKER_OK) return rc;
    if (!max_given) CUDA_TRY(cudaMemsetAsync(d_exact_key, 0, sizeof(uint64_t) * n_slots, st));
    a.write_max = 1;
    a.u_source = u_source;
    a.u = d_u;
    a.out_idx = d_out_idx;
    a.out_lnl = d_out_lnl;
    a.count = d_count;
    CUDA_TRY(launch_accept(a, nb, st, max_given != 0));
    return JOKER_OK;
}

extern "C" int joker_accept_fused(const joker_stars *s, const joker_cache *c,
                                  const joker_accept_seg *segs, int n_segs, double *d_lnl,
                                  float *d_err, const uint64_t *d_bound_key,
                                  uint64_t *d_exact_key, int n_slots, const uint32_t *d_cand,
                                  int64_t cand_ld, int64_t *d_out_idx, double *d_out_lnl,
                                  int64_t *d_count, uint64_t *d_n_refined, void *d_work,
                                  int64_t work_bytes, void *stream) {
    if (n_segs <= 0) return JOKER_OK;
    if (!d_out_idx || !d_count || !d_cand)
        return fail(JOKER_EINVAL, "joker_accept_fused: NULL argument");
    if (cand_ld % 4 || ((uintptr_t)d_cand) % 16)
        return fail(JOKER_EINVAL, "joker_accept_fused: cand_ld must be a multiple of 4 and "
                                  "d_cand 16-byte aligned");
    if (segs)
        for (int i = 0; i < n_segs; ++i)
            if (segs[i].n > 32 * cand_ld)
                return fail(JOKER_EINVAL, "joker_accept_fused: segment %d has %lld samples, "
                                          "cand_ld %lld words", i, (long long)segs[i].n,
                            (long long)cand_ld);
    AcceptArgs a;
    int64_t nb = 0;
    cudaStream_t st = (cudaStream_t)stream;
    const int rc = refined_setup(s, c, segs, n_segs, d_lnl, d_err, d_bound_key, d_exact_key,
                                 n_slots, d_n_refined, d_work, work_bytes, st, a, nb,
                                 "joker_accept_fused");
    if (rc != JOKER_OK) return rc;
    CUDA_TRY(cudaMemsetAsync(d_exact_key, 0, sizeof(uint64_t) * n_slots, st));
    a.write_max = 1;
    a.u_source = JOKER_U_PCG64;
    a.out_idx = d_out_idx;
    a.out_lnl = d_out_lnl;
    a.count = d_count;
    a.cand_words = d_cand;
    a.cand_ld = cand_ld;
    CUDA_TRY(launch_accept_fused(a, nb, st));
    return JOKER_OK;
}

// ------------------------------------------------- one-call rejection step
// The sequence the host engines run, as one entry: ln L of every (star,
// sample), the running maxima, and the acceptance against each star's PCG64
// stream, refined to FP64 decisions for the mixed precisions.
static void rejection_segs(int star0, int n_sel, int64_t row0, int64_t count, int64_t max_out,
                           const uint64_t *pcg, std::vector<joker_accept_seg> &segs) {
    segs.assign(n_sel, joker_accept_seg{});
    for (int k = 0; k < n_sel; ++k) {
        joker_accept_seg &g = segs[k];
        g.lnl_off = (int64_t)k * count;
        g.n = count;
        g.idx_base = row0;
        g.out_off = (int64_t)k * max_out;
        g.max_out = max_out;
        g.u_off = 0;
        if (pcg) {
            g.pcg_state_hi = pcg[4 * k + 0];
            g.pcg_state_lo = pcg[4 * k + 1];
            g.pcg_inc_hi = pcg[4 * k + 2];
            g.pcg_inc_lo = pcg[4 * k + 3];
        }
        g.max_slot = k;
        g.star = star0 + k;
        g.row0 = row0;
    }
}

// Scratch layout: ln L (n_sel x count doubles), bounds (n_sel x count
// floats, mixed only), 4 n_sel keys (running maxima, two bound maxima,
// FP64 maxima); for JOKER_MIXED_FAST the generator states (4 words per star)
// and the fused pass's candidate bits (cand_ld words per star); then the
// acceptance workspace.
struct RejLayout {
    int64_t err, keys, pcg, cand, acc, total, cand_ld;
};

static RejLayout rejection_layout(int n_sel, int64_t count, int64_t max_out, int precision) {
    std::vector<joker_accept_seg> segs;
    rejection_segs(0, n_sel, 0, count, max_out, nullptr, segs);
    RejLayout r;
    const int64_t lnl = align256(8 * (int64_t)n_sel * count);
    const int64_t err = precision == JOKER_FP64 ? 0 : align256(4 * (int64_t)n_sel * count);
    const int64_t keys = align256(8 * 4 * (int64_t)n_sel);
    const bool fused = precision == JOKER_MIXED_FAST;
    r.cand_ld = ((count + 31) / 32 + 7) & ~(int64_t)7;
    const int64_t pcg = fused ? align256(32 * (int64_t)n_sel) : 0;
    const int64_t cand = fused ? align256(4 * r.cand_ld * (int64_t)n_sel) : 0;
    r.err = lnl;
    r.keys = lnl + err;
    r.pcg = r.keys + keys;
    r.cand = r.pcg + pcg;
    r.acc = r.cand + cand;
    r.total = r.acc + joker_accept_workspace(segs.data(), n_sel);
    return r;
}

extern "C" int64_t joker_rejection_workspace(int n_sel, int64_t count, int64_t max_out,
                                             int precision) {
    if (n_sel <= 0 || count <= 0 || max_out < 0) return 0;
    return rejection_layout(n_sel, count, max_out, precision).total;
}

extern "C" int joker_rejection_sample(const joker_stars *s, const joker_cache *c, int star0,
                                      int n_sel, int64_t row0, int64_t count, int precision,
                                      const uint64_t *pcg, int64_t max_out, int64_t *d_out_idx,
                                      double *d_out_lnl, int64_t *d_count, void *d_work,
                                      int64_t work_bytes, void *stream) {
    if (!s || !c) return fail(JOKER_EINVAL, "joker_rejection_sample: NULL handle");
    if (n_sel < 0 || count < 0 || max_out < 0)
        return fail(JOKER_EINVAL, "joker_rejection_sample: negative size");
    if (n_sel == 0 || count == 0) return JOKER_OK;
    if (!pcg || !d_out_idx || !d_count || !d_work)
        return fail(JOKER_EINVAL, "joker_rejection_sample: NULL argument");
    const RejLayout lay = rejection_layout(n_sel, count, max_out, precision);
    if (work_bytes < lay.total)
        return fail(JOKER_EINVAL, "joker_rejection_sample: workspace %lld bytes, needs %lld",
                    (long long)work_bytes, (long long)lay.total);
    if (((uintptr_t)d_work) % 256)
        return fail(JOKER_EINVAL, "joker_rejection_sample: workspace not 256-byte aligned");
    char *w = (char *)d_work;
    double *lnl = (double *)w;
    float *err = precision == JOKER_FP64 ? nullptr : (float *)(w + lay.err);
    uint64_t *keys = (uint64_t *)(w + lay.keys);
    uint64_t *max_key = keys, *bound_key = keys + n_sel, *exact_key = keys + 3 * n_sel;
    cudaStream_t st = (cudaStream_t)stream;
    CUDA_TRY(cudaMemsetAsync(keys, 0, 8 * 4 * (size_t)n_sel, st));
    std::vector<joker_accept_seg> segs;
    rejection_segs(star0, n_sel, row0, count, max_out, pcg, segs);
    const int64_t acc_bytes = work_bytes - lay.acc;
    // JOKER_MIXED_FAST: the first acceptance pass fused into the ln L kernel
    // (a jittered table with more than three linear parameters runs the
    // float-float kernel and the separate passes instead)
    if (precision == JOKER_MIXED_FAST && !(s->jitter == JOKER_JITTER_APPLIED && s->L > 3)) {
        uint64_t *d_pcg = (uint64_t *)(w + lay.pcg);
        uint32_t *cand = (uint32_t *)(w + lay.cand);
        CUDA_TRY(cudaMemcpyAsync(d_pcg, pcg, 32 * (size_t)n_sel, cudaMemcpyHostToDevice, st));
        int rc = joker_lnl_fused(s, c, star0, n_sel, row0, count, d_pcg, 0, lnl, count, max_key,
                                 err, bound_key, cand, lay.cand_ld, 0, 0, stream);
        if (rc != JOKER_OK) return rc;
        return joker_accept_fused(s, c, segs.data(), n_sel, lnl, err, bound_key, exact_key,
                                  n_sel, cand, lay.cand_ld, d_out_idx, d_out_lnl, d_count,
                                  nullptr, w + lay.acc, acc_bytes, stream);
    }
    int rc = joker_lnl(s, c, star0, n_sel, row0, count, precision, lnl, count, max_key, err,
                       bound_key, 0, 0, stream);
    if (rc != JOKER_OK) return rc;
    if (precision == JOKER_FP64)
        return joker_accept(segs.data(), n_sel, lnl, max_key, JOKER_U_PCG64, nullptr, d_out_idx,
                            d_out_lnl, d_count, w + lay.acc, acc_bytes, stream);
    return joker_accept_refined(s, c, segs.data(), n_sel, lnl, err, bound_key, exact_key, n_sel, 0,
                                JOKER_U_PCG64, nullptr, d_out_idx, d_out_lnl, d_count, nullptr,
                                w + lay.acc, acc_bytes, stream);
}
