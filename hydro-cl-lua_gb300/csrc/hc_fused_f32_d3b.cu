// hc_fused_f32_d3b.cu -- 3D stage kernels, FP32 (fast form): smaller tiles at
// 128 registers a thread and 4 CTAs per SM, the sliding window unrolled by 2.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d3b(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    (void)aux;
    // 4: 8x8x8, segments of 4, 128 threads
    // 5: 16x8x4, segments of 4, 128 threads
    add_plm_set<T, P, 3, 4, 8, 8, 8, 4, 128, 2, 4>(st);
    add_plm_set<T, P, 3, 5, 16, 8, 4, 4, 128, 2, 4>(st);
}

}  // namespace fz
}  // namespace hc
