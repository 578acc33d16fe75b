// Launchers of the FP32-sum ln L kernel (JOKER_MIXED_FAST), in both of its
// forms: reading the prepared cache, or packed FP64 rows prepared in
// registers (cache views).  Any number of linear parameters without the
// jitter; at most three with it (launch_lnl routes larger jittered systems
// to the float-float kernel).
#include "joker_fast.cuh"

namespace joker {

template <int L, bool JIT>
static cudaError_t launch_fast_LJ(const LnlArgs &a, int block, cudaStream_t st) {
    if (a.mx_a == nullptr) return launch_persistent(lnl_fast2_kernel<L, JIT, true>, a, block, st);
    return launch_persistent(lnl_fast2_kernel<L, JIT, false>, a, block, st);
}

cudaError_t launch_lnl_fast(int L, bool jit, const LnlArgs &a, int block, cudaStream_t st) {
    if (jit) {
        switch (L) {
            case 1: return launch_fast_LJ<1, true>(a, block, st);
            case 2: return launch_fast_LJ<2, true>(a, block, st);
            case 3: return launch_fast_LJ<3, true>(a, block, st);
        }
        return cudaErrorInvalidValue;
    }
    switch (L) {
        case 1: return launch_fast_LJ<1, false>(a, block, st);
        case 2: return launch_fast_LJ<2, false>(a, block, st);
        case 3: return launch_fast_LJ<3, false>(a, block, st);
        case 4: return launch_fast_LJ<4, false>(a, block, st);
        case 5: return launch_fast_LJ<5, false>(a, block, st);
        case 6: return launch_fast_LJ<6, false>(a, block, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace joker
