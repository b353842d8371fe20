// hc_fused_f32_m2b.cu -- more 2D marching schedules (hc_march.cuh): the
// 3-CTA-per-SM kernel of schedule 17 with the limiters of the other
// configurations compiled in, and with shorter segments.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_m2b(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    (void)aux;
    add_march2<17, 4, 64, 8, 2, HC_LIMITER_MONOTIZED_CENTRAL, 3>(st);
    add_march2<17, 4, 64, 8, 2, HC_LIMITER_MINMOD, 3>(st);
    // 19: as 17 with segments of 16 rows, for grids too few to fill the GPU
    // with 64-row segments (one 1024^2 grid: 560 segments of 64 rows for 1824
    // resident warps; 2240 of 16 rows)
    add_march2<19, 4, 16, 8, 2, -1, 3>(st);
    add_march2<19, 4, 16, 8, 2, HC_LIMITER_MONOTIZED_CENTRAL, 3>(st);
    add_march2<19, 4, 16, 8, 2, HC_LIMITER_VAN_LEER_ABS, 3>(st);
    add_march2<19, 4, 16, 8, 2, HC_LIMITER_MINMOD, 3>(st);
    // 20: segments of 32 rows
    add_march2<20, 4, 32, 8, 2, -1, 3>(st);
    add_march2<20, 4, 32, 8, 2, HC_LIMITER_MONOTIZED_CENTRAL, 3>(st);
    add_march2<20, 4, 32, 8, 2, HC_LIMITER_VAN_LEER_ABS, 3>(st);
}

}  // namespace fz
}  // namespace hc
