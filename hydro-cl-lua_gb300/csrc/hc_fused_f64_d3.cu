// hc_fused_f64_d3.cu -- 3D stage kernels, FP64 (exact form, no FMA contraction).
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f64_d3(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = double;
    constexpr int P = HC_F64_FUSED;
    constexpr bool E = true;
    add_stage<T, P, 3, 0, 16, 8, 8, 8, 128, E, -1, false>(st);
    add_stage<T, P, 3, 0, 16, 8, 8, 8, 128, E, 0, false>(st);
    add_stage<T, P, 3, 0, 16, 8, 8, 8, 128, E, 0, true>(st);
    add_aux<T, P, 3, E>(aux);
}

}  // namespace fz
}  // namespace hc
