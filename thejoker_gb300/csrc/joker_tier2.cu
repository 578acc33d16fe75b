// The middle tier of the refined acceptance: the candidates for a star's FP64
// maximum (flag list 0 after the candidates scan) re-evaluated with the
// float-float kernel's arithmetic before any FP64 work.
//
// The FP32-sum first pass (JOKER_MIXED_FAST) states bounds of up to hundreds
// of nats for poorly fitting samples, so its candidate list can hold 10^5
// samples of a 2^28 cache; the float-float sums tighten each interval to its
// column error, raise the star's largest lower bound, and leave for FP64 only
// the samples whose tightened interval still reaches it.  One thread per
// listed sample, the star's epoch records read from global memory (they stay
// in L1/L2 for the few stars of a pass); a sample keeps its old value and
// bound unless the new bound is tighter.
#include "joker_mixed.cuh"

namespace joker {

// Entries whose bound is already at most this are left as they are (the
// float-float bound is not smaller); entries without a bound (err >= 1e29,
// the FP32-sum bound's validity test failed) are re-evaluated like the rest.
constexpr float TIER2_MIN_ERR = 1e-6f;

template <int L, bool JIT>
__global__ void __launch_bounds__(128) tier2_kernel(AcceptArgs a) {
    const int64_t n = min((int64_t)a.flag_count[0], a.flag_cap);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ent = a.flag_list[e];
        const int si = (int)(ent >> 40);
        const int64_t i = ent & (((int64_t)1 << 40) - 1);
        const joker_accept_seg sg = a.segs[si];
        const int64_t o = sg.lnl_off + i;
        const float er0 = a.err[o];
        if (!(er0 > TIER2_MIN_ERR)) continue;                // exact, tight, or NaN
        const int64_t r = (sg.row0 + i) * a.stride;
        float4 pa, pb;
        float s2;
        prepare_sample(a.P[r], a.E[r], a.OM[r], a.M0[r], JIT ? a.S[r] : 0.0, pa, pb, s2);
        const StarRec &st = a.stars[sg.star];
        const MixC<float> c = mix_consts(pa, pb, s2);
        Acc32<L, JIT, float> A;
        A.zero();
        const float *rec = a.ep32 + (size_t)st.epoch_off * REC32;
        const bool mu0z = st.mu0_zero != 0;
        for (int k = 0; k < st.n_epochs; ++k)
            mixed_epoch<L, JIT, false>(rec + (size_t)k * REC32, c, mu0z, st.mu0_f, -st.mu0_f, A);
        double v;
        float er;
        mixed_tail<L, JIT, 0>(st, A, c.e, c.ome, pb.w, st.n_epochs, a.err_c0, v, er);
        if (er < er0) {
            const_cast<double *>(a.lnl)[o] = v;
            const_cast<float *>(a.err)[o] = er;
            atomicMax(const_cast<unsigned long long *>(a.bound_key) + 2 * sg.max_slot + 1,
                      double_to_key(v - (double)er));
        }
    }
}

template <int L>
static void launch_tier2_L(const AcceptArgs &a, cudaStream_t st) {
    if (a.jit) tier2_kernel<L, true><<<152 * 8, 128, 0, st>>>(a);
    else tier2_kernel<L, false><<<152 * 8, 128, 0, st>>>(a);
}

cudaError_t launch_tier2(const AcceptArgs &a, cudaStream_t st) {
    switch (a.L) {
        case 1: launch_tier2_L<1>(a, st); break;
        case 2: launch_tier2_L<2>(a, st); break;
        case 3: launch_tier2_L<3>(a, st); break;
        case 4: launch_tier2_L<4>(a, st); break;
        case 5: launch_tier2_L<5>(a, st); break;
        case 6: launch_tier2_L<6>(a, st); break;
        default: return cudaErrorInvalidValue;
    }
    count_launch();
    return cudaGetLastError();
}

}  // namespace joker
