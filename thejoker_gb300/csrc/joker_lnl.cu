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
#include "joker_mixed.cuh"

namespace joker {

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
        float4 pa, pb;
        float s2;
        prepare_sample(p, e, om, m0, s, pa, pb, s2);
        mx_a[r] = pa;
        mx_b[r] = pb;
        mx_s2[r] = s2;
    }
}

// ------------------------------------------------------------------ launchers
cudaError_t launch_lnl_packed(int precision, int L, bool jit, const LnlArgs &a, int block,
                              cudaStream_t st);

template <int L>
static cudaError_t launch_fp64_L(bool jit, const LnlArgs &a, int block, cudaStream_t st) {
    if (jit) return launch_persistent(lnl_fp64_kernel<L, true>, a, block, st);
    return launch_persistent(lnl_fp64_kernel<L, false>, a, block, st);
}

template <int L, int VAR>
static cudaError_t launch_mixed_LV(bool jit, const LnlArgs &a, int block, cudaStream_t st) {
    if (mixed_paired(L, jit)) {
        if constexpr (L <= 3) {
            if (jit) return launch_persistent(lnl_mixed2_kernel<L, true, VAR, false>, a, block, st);
        }
        return launch_persistent(lnl_mixed2_kernel<L, false, VAR, false>, a, block, st);
    }
    if (jit) return launch_persistent(lnl_mixed_kernel<L, true, VAR, false>, a, block, st);
    return launch_persistent(lnl_mixed_kernel<L, false, VAR, false>, a, block, st);
}

template <int L>
static cudaError_t launch_mixed_L(bool jit, int var, const LnlArgs &a, int block,
                                  cudaStream_t st) {
    if (var == 1) return launch_mixed_LV<L, 1>(jit, a, block, st);
    if (var == 2) return launch_mixed_LV<L, 2>(jit, a, block, st);
    return launch_mixed_LV<L, 0>(jit, a, block, st);
}

cudaError_t launch_lnl_fast(int L, bool jit, const LnlArgs &a, int block, cudaStream_t st);

cudaError_t launch_lnl(int precision, int L, bool jit, const LnlArgs &a, int block,
                       cudaStream_t st) {
    // The FP32-sum kernel covers any number of linear parameters without the
    // jitter and at most three with it; larger jittered systems run the
    // float-float kernel, whose outputs are of the same kind (tighter bound).
    if (precision == JOKER_MIXED_FAST) {
        if (!jit || L <= 3) return launch_lnl_fast(L, jit, a, block, st);
        precision = JOKER_MIXED;
    }
    if (precision == JOKER_FP64) {
        switch (L) {
            case 1: return launch_fp64_L<1>(jit, a, block, st);
            case 2: return launch_fp64_L<2>(jit, a, block, st);
            case 3: return launch_fp64_L<3>(jit, a, block, st);
            case 4: return launch_fp64_L<4>(jit, a, block, st);
            case 5: return launch_fp64_L<5>(jit, a, block, st);
            case 6: return launch_fp64_L<6>(jit, a, block, st);
        }
    } else if (a.mx_a == nullptr) {
        return launch_lnl_packed(precision, L, jit, a, block, st);
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
    count_launch();
    return cudaGetLastError();
}

}  // namespace joker
