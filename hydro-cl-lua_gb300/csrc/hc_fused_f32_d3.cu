// hc_fused_f32_d3.cu -- 3D stage kernels, FP32 (fast form).
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d3(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    constexpr bool E = false;
    // variants: 0: 16x8x8, segments of 4, 256 threads; 1: 32x8x8, segments of 8, 256 threads;
    //           2: 16x8x8, segments of 8, 128 threads
    add_plm_set<T, P, 3, 0, 16, 8, 8, 4, 256>(st);
    add_plm_set<T, P, 3, 1, 32, 8, 8, 8, 256>(st);
    add_plm_pair<T, P, 3, 2, 16, 8, 8, 8, 128, 0>(st);
    // 3: 16x8x8, segments of 4, 256 threads, 1 CTA per SM (255 registers)
    add_plm_set<T, P, 3, 3, 16, 8, 8, 4, 256, 0, 1>(st);
    add_stage<T, P, 3, 0, 16, 8, 8, 4, 256, E, 0, false>(st);
    add_stage<T, P, 3, 0, 16, 8, 8, 4, 256, E, 0, true>(st);
    add_aux<T, P, 3, E>(aux);
}

}  // namespace fz
}  // namespace hc
