/*
 * rsc_step.cuh -- one pass over the state per pulse.
 *
 * simradar's loop is make_pulse(k), advance(k), make_pulse(k + 1), ...  The
 * pulse k + 1 reads exactly the positions and backscatter that advance(k)
 * writes, so the step kernel advances each scatterer and adds it to pulse
 * k + 1 from registers: the state is read and written once per pulse instead
 * of read again by a separate pulse kernel.  The grid is persistent (a few
 * blocks per SM, each looping over the advance's blocks of kAdvanceThreads scatterers)
 * so that every block's gate bins are added to the FP64 accumulator once.
 * Results are those of the advance kernels followed by k_pulse: the same per-scatterer
 * operations, the gate sums in another order.
 */
#ifndef SIMRADAR_GB300_RSC_STEP_CUH
#define SIMRADAR_GB300_RSC_STEP_CUH

#include "rsc_pulse.cuh"

namespace rsc {

template <int MODE>
__device__ __forceinline__ void step_body(const AdvanceArgs &a, const PulseArgs &P, unsigned vblocks, unsigned blk,
                                          unsigned nblk) {
    PulseBins<MODE> B;
    B.init(P);
    for (unsigned vb = blk; vb < vblocks; vb += nblk) {
        unsigned long long i = 0;
        float4 pos = make_float4(0.0f, 0.0f, 0.0f, 0.0f), rcs = pos;
        const bool in = advance_one(a, vb, i, pos, rcs);
        B.add(P, in, i, pos, rcs);
    }
    B.finish(P, nblk);
}

template <int MODE>
__global__ void __launch_bounds__(kAdvanceThreads) k_step(const AdvanceArgs a, const PulseArgs P, unsigned vblocks) {
    step_body<MODE>(a, P, vblocks, blockIdx.x, gridDim.x);
}

}  // namespace rsc

#endif
