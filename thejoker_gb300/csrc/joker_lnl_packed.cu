// The mixed ln L kernel in its packed form: samples read as FP64 rows of the
// reference's (S, 5) chunk (P, e, omega, M0, s; a.stride doubles apart) and
// prepared in registers.  Used for a cache view (joker_cache_create_view)
// over a chunk in device memory or in mapped pinned host memory, where it
// saves the separate preparation pass and, for host memory, the staging copy.
#include "joker_mixed.cuh"

namespace joker {

template <int L, int VAR>
static cudaError_t launch_packed_LV(bool jit, const LnlArgs &a, int block, cudaStream_t st) {
    if (mixed_paired(L, jit)) {
        if constexpr (L <= 3) {
            if (jit) return launch_persistent(lnl_mixed2_kernel<L, true, VAR, true>, a, block, st);
        }
        return launch_persistent(lnl_mixed2_kernel<L, false, VAR, true>, a, block, st);
    }
    if (jit) return launch_persistent(lnl_mixed_kernel<L, true, VAR, true>, a, block, st);
    return launch_persistent(lnl_mixed_kernel<L, false, VAR, true>, a, block, st);
}

template <int L>
static cudaError_t launch_packed_L(bool jit, int var, const LnlArgs &a, int block,
                                   cudaStream_t st) {
    if (var == 1) return launch_packed_LV<L, 1>(jit, a, block, st);
    if (var == 2) return launch_packed_LV<L, 2>(jit, a, block, st);
    return launch_packed_LV<L, 0>(jit, a, block, st);
}

cudaError_t launch_lnl_packed(int precision, int L, bool jit, const LnlArgs &a, int block,
                              cudaStream_t st) {
    const int var = precision == JOKER_MIXED_ACCURATE ? 1
                  : precision == JOKER_MIXED_FP64_TAIL ? 2 : 0;
    switch (L) {
        case 1: return launch_packed_L<1>(jit, var, a, block, st);
        case 2: return launch_packed_L<2>(jit, var, a, block, st);
        case 3: return launch_packed_L<3>(jit, var, a, block, st);
        case 4: return launch_packed_L<4>(jit, var, a, block, st);
        case 5: return launch_packed_L<5>(jit, var, a, block, st);
        case 6: return launch_packed_L<6>(jit, var, a, block, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace joker
