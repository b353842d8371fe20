// hc_fused_f32_m2.cu -- 2D marching stage kernels (hc_march.cuh), FP32 fast
// form, "plm cons" with the Roe flux: one warp per 30-column strip marching up
// a segment of rows.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_m2(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    (void)aux;
    // 16: 4 warps per CTA, segments of 64 rows, chunks of 8 rows double-buffered, 4 CTAs per SM
    add_march2<16, 4, 64, 8, 2, -1, 4>(st);
    add_march2<16, 4, 64, 8, 2, HC_LIMITER_MINMOD, 4>(st);
    add_march2<16, 4, 64, 8, 2, HC_LIMITER_MONOTIZED_CENTRAL, 4>(st);
    add_march2<16, 4, 64, 8, 2, HC_LIMITER_VAN_LEER_ABS, 4>(st);
    add_march2<16, 4, 64, 8, 2, HC_LIMITER_SUPERBEE, 4>(st);
    // 17: as 16 at 3 CTAs per SM (168 registers a thread); 18: at 2 CTAs per SM
    add_march2<17, 4, 64, 8, 2, -1, 3>(st);
    add_march2<17, 4, 64, 8, 2, HC_LIMITER_VAN_LEER_ABS, 3>(st);
    add_march2<18, 4, 64, 8, 2, -1, 2>(st);
    add_march2<18, 4, 64, 8, 2, HC_LIMITER_VAN_LEER_ABS, 2>(st);
}

}  // namespace fz
}  // namespace hc
