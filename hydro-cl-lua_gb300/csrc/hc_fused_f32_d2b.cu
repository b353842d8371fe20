// hc_fused_f32_d2b.cu -- 2D stage kernels, FP32 (fast form): the kernels
// without reconstruction (plain and flux-limited Roe) and the auxiliary ones.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d2b(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    constexpr bool E = false;
    add_stage<T, P, 2, 0, 32, 32, 1, 4, 256, E, 0, false>(st);
    add_stage<T, P, 2, 0, 32, 32, 1, 4, 256, E, 0, true>(st);
    add_aux<T, P, 2, E>(aux);
}

}  // namespace fz
}  // namespace hc
