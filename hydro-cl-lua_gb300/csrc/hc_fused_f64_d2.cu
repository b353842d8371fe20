// hc_fused_f64_d2.cu -- 2D stage kernels, FP64 (exact form, no FMA contraction).
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f64_d2(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = double;
    constexpr int P = HC_F64_FUSED;
    constexpr bool E = true;
    add_stage<T, P, 2, 0, 32, 32, 1, 8, 128, E, -1, false>(st);
    add_stage<T, P, 2, 0, 32, 32, 1, 8, 128, E, 0, false>(st);
    add_stage<T, P, 2, 0, 32, 32, 1, 8, 128, E, 0, true>(st);
    add_aux<T, P, 2, E>(aux);
}

}  // namespace fz
}  // namespace hc
