// Launchers of the FP32-sum ln L kernel (JOKER_MIXED_FAST), in both of its
// forms: reading the prepared cache, or packed FP64 rows prepared in
// registers (cache views).  Any number of linear parameters without the
// jitter; at most three with it (launch_lnl routes larger jittered systems
// to the float-float kernel).
#include "joker_fast.cuh"

namespace joker {

cudaError_t launch_lnl_fast(int L, bool jit, const LnlArgs &a, int block, cudaStream_t st) {
    return launch_fast_any<false>(L, jit, a, block, st);
}

}  // namespace joker
