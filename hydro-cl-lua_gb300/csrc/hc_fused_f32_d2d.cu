// hc_fused_f32_d2d.cu -- 2D stage kernels, FP32 (fast form): schedules that
// trade resident CTAs for registers or unrolling for a smaller instruction
// footprint, for the autotuner to weigh against the primary ones.
//
// Schedules sweeping two lines per thread with packed FP32 pairs (LANES = 2)
// compile from the same template but are not registered: on the batched
// quadrant workload they issue 31 % fewer instructions per cell, yet need
// twice the registers per thread (half the resident warps) and a larger
// instruction footprint, and ran 9-60 % slower per stage than the best
// one-line schedule; they also round the flux differently from the one-line
// kernels in the last bit at some interfaces.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d2d(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    (void)aux;
    // 7: 32x32, segments of 4, 256 threads, 3 CTAs per SM (85 registers)
    // 8: 32x32, segments of 4, 256 threads, rolled sliding window (smaller footprint)
    // 9: 32x64, segments of 8, 256 threads, rolled sliding window
    add_plm_pair<T, P, 2, 7, 32, 32, 1, 4, 256, 0, 3>(st);
    add_plm_pair<T, P, 2, 8, 32, 32, 1, 4, 256, 1>(st);
    add_plm_pair<T, P, 2, 9, 32, 64, 1, 8, 256, 1>(st);
}

}  // namespace fz
}  // namespace hc
