// hc_fused_f32_d3c.cu -- 3D stage kernels, FP32 (fast form): the 16x8x8 tile
// of schedule 0 (segments of 4, 256 threads, 2 CTAs per SM) with the sliding
// window unrolled by 2 instead of fully: a smaller instruction footprint (the
// fully unrolled kernel's top stall is instruction fetch).  On the 256^3
// blast: 1.786 ms per step against 1.837 (the window rolled: 1.793).
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d3c(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    (void)aux;
    // 6: 16x8x8, segments of 4, 256 threads, window unrolled by 2
    add_plm_set<T, P, 3, 6, 16, 8, 8, 4, 256, 2>(st);
}

}  // namespace fz
}  // namespace hc
