// hc_fused_f32_d2c.cu -- 2D stage kernels, FP32 (fast form): further
// schedules timed by the autotuner (segment length, unrolling, tile shape),
// for the batched configuration's limiter and the generic one.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d2c(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    (void)aux;
    // 2: 64x32, segments of 8, 256 threads, unrolled by 2
    // 3: 64x32, segments of 8, 256 threads, fully unrolled
    // 4: 64x16, segments of 4, 256 threads
    // 5: 32x64, segments of 4, 512 threads
    // 6: 32x32, segments of 4, 256 threads, unrolled by 2
    add_plm_pair<T, P, 2, 2, 64, 32, 1, 8, 256, 2>(st);
    add_plm_pair<T, P, 2, 3, 64, 32, 1, 8, 256, 0>(st);
    add_plm_pair<T, P, 2, 4, 64, 16, 1, 4, 256, 0>(st);
    add_plm_pair<T, P, 2, 5, 32, 64, 1, 4, 512, 0>(st);
    add_plm_pair<T, P, 2, 6, 32, 32, 1, 4, 256, 2>(st);
}

}  // namespace fz
}  // namespace hc
