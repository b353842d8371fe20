// hc_fused_f32_d2d.cu -- 2D stage kernels, FP32 (fast form): schedules that
// sweep two lines per thread with packed FP32 pairs, and schedules that trade
// resident CTAs for registers, for the autotuner to weigh against the
// primary ones.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d2d(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    (void)aux;
    // 7: 32x32, segments of 4, 256 threads, 3 CTAs per SM (85 registers)
    // 8: 32x32, segments of 4, 128 threads, two lines per thread
    // 9: 32x32, segments of 8, 128 threads, two lines per thread, unrolled by 2
    // 10: 64x32, segments of 4, 256 threads, two lines per thread
    add_plm_pair<T, P, 2, 7, 32, 32, 1, 4, 256, 0, 3>(st);
    add_plm_pair<T, P, 2, 8, 32, 32, 1, 4, 128, 0, 0, 2>(st);
    add_plm_pair<T, P, 2, 9, 32, 32, 1, 8, 128, 2, 0, 2>(st);
    add_plm_pair<T, P, 2, 10, 64, 32, 1, 4, 256, 0, 0, 2>(st);
}

}  // namespace fz
}  // namespace hc
