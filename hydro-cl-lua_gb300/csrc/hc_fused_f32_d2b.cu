// hc_fused_f32_d2b.cu -- 2D stage kernels, FP32 (fast form): PLM tile variants 2 and 3, the others.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d2b(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    constexpr bool E = false;
    // variants: 64x16 (128 thr), 128x16 (256 thr); L = 8
    add_plm_set<T, P, 2, 2, 64, 16, 1, 8, 128>(st);
    add_plm_set<T, P, 2, 3, 128, 16, 1, 8, 256>(st);
    add_stage<T, P, 2, 0, 64, 32, 1, 8, 256, E, false, false>(st);
    add_stage<T, P, 2, 0, 64, 32, 1, 8, 256, E, false, true>(st);
    add_aux<T, P, 2, E>(aux);
}

}  // namespace fz
}  // namespace hc
