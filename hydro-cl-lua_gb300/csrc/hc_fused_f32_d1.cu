// hc_fused_f32_d1.cu -- 1D stage kernels, FP32 (fast form).
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d1(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    constexpr bool E = false;
    // variants: tile 128 x (L 4, 32 threads); tile 64 x (L 2, 32 threads)
    add_plm_set<T, P, 1, 0, 128, 1, 1, 4, 32>(st);
    add_plm_set<T, P, 1, 1, 64, 1, 1, 2, 32>(st);
    add_stage<T, P, 1, 0, 128, 1, 1, 4, 32, E, 0, false>(st);
    add_stage<T, P, 1, 0, 128, 1, 1, 4, 32, E, 0, true>(st);
    add_aux<T, P, 1, E>(aux);
}

}  // namespace fz
}  // namespace hc
