// hc_fused_f32_d2c.cu -- 2D stage kernels, FP32 (fast form): extra schedules
// (shorter segments for more resident warps, partial unrolling for a smaller
// code footprint) timed by the autotuner.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d2c(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    (void)aux;
    // 4: 64x32, L 4, 512 threads; 5: 64x32, L 8, unroll 2; 6: 64x32, L 4, 512 threads, unroll 2;
    // 7: 32x32, L 4, 256 threads
    add_plm_pair<T, P, 2, 4, 64, 32, 1, 4, 512, 0>(st);
    add_plm_pair<T, P, 2, 5, 64, 32, 1, 8, 256, 2>(st);
    add_plm_pair<T, P, 2, 6, 64, 32, 1, 4, 512, 2>(st);
    add_plm_pair<T, P, 2, 7, 32, 32, 1, 4, 256, 0>(st);
}

}  // namespace fz
}  // namespace hc
