// hc_fused_f32_d2a.cu -- 2D stage kernels, FP32 (fast form): the primary PLM
// schedules, every compiled-in slope limiter.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d2a(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    (void)aux;
    // 0: 32x32 tile, segments of 4, 256 threads; 1: 64x32, segments of 4, 512 threads
    add_plm_set<T, P, 2, 0, 32, 32, 1, 4, 256>(st);
    add_plm_set<T, P, 2, 1, 64, 32, 1, 4, 512>(st);
}

}  // namespace fz
}  // namespace hc
