// split_rows4_128.cu -- the split form's vector row kernel at N = 128: every
// launch shape (one step per launch, and persistent) of both potentials.
#include "split_rows4.cuh"

namespace iegpu {

void rows4_launch_128(iegpu_ctx* c, bool tab, const SplitBufs& B, const SplitConst& K, dim3 grid, const StepGeom& g) {
    if (tab) rows4_tj<true, 1>(c, B, K, grid, g);
    else rows4_tj<false, 1>(c, B, K, grid, g);
}

int rows4_persist_128(iegpu_ctx* c, bool tab, int start, int nsteps, dim3 grid, const StepGeom& g, bool check_only) {
    return tab ? persist_tj<true, 1>(c, start, nsteps, grid, g, check_only)
               : persist_tj<false, 1>(c, start, nsteps, grid, g, check_only);
}

}  // namespace iegpu
