// hc_fused_f32_d2a.cu -- 2D stage kernels, FP32 (fast form): PLM tile variants 0 and 1.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d2a(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    constexpr bool E = false;
    (void)E;
    (void)aux;
    // variants: 64x32 (256 thr), 32x32 (128 thr); L = 8
    add_plm_set<T, P, 2, 0, 64, 32, 1, 8, 256>(st);
    add_plm_set<T, P, 2, 1, 32, 32, 1, 8, 128>(st);
}

}  // namespace fz
}  // namespace hc
