// Launchers of the FP32-sum ln L kernel with the fused first acceptance pass
// (each sample's PCG64 uniform and candidate bit written beside its ln L).
// Same forms and limits as joker_lnl_fast.cu; a translation unit of its own
// so that the two sets of instances compile in parallel.
#include "joker_fast.cuh"

namespace joker {

cudaError_t launch_lnl_fused(int L, bool jit, const LnlArgs &a, int block, cudaStream_t st) {
    return launch_fast_any<true>(L, jit, a, block, st);
}

}  // namespace joker
