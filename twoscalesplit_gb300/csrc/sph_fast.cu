// sph_fast.cu -- the gathers in the tolerance arithmetic (gathers.cuh with
// FastArith, arith.cuh): selected per handle by tss_solver_set_arith.
#include "gathers.cuh"

namespace tss {

void launch_gather_fast(int g, bool batched, bool warp, int blocks, int threads, cudaStream_t s, const Params& P,
                        const StepView& V) {
    launch_gather_a<FastArith>(g, batched, warp, blocks, threads, s, P, V);
}

int gather_occupancy_fast(int g, bool batched, bool warp, int threads) {
    return gather_occupancy_a<FastArith>(g, batched, warp, threads);
}

}  // namespace tss
