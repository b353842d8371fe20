// hc_fused_f32_m3.cu -- 3D marching stage kernels (hc_march3.cuh), FP32 fast
// form, "plm cons" with the Roe flux: one CTA per x-y tile marching up a
// segment of planes along z.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_m3(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    (void)aux;
    // 7: 12 warps (30 x 11 tiles), segments of 32 planes, 5 plane buffers, 1 CTA per SM
    add_march3<7, 12, 32, 5, -1, 1>(st);
    add_march3<7, 12, 32, 5, HC_LIMITER_MINMOD, 1>(st);
    add_march3<7, 12, 32, 5, HC_LIMITER_MONOTIZED_CENTRAL, 1>(st);
    add_march3<7, 12, 32, 5, HC_LIMITER_VAN_LEER_ABS, 1>(st);
    add_march3<7, 12, 32, 5, HC_LIMITER_SUPERBEE, 1>(st);
    // 8: as 7 with segments of 64 planes
    add_march3<8, 12, 64, 5, -1, 1>(st);
    add_march3<8, 12, 64, 5, HC_LIMITER_MINMOD, 1>(st);
    // 9: 16 warps (30 x 15 tiles), 1 CTA per SM (128 registers a thread)
    add_march3<9, 16, 32, 5, -1, 1>(st);
    add_march3<9, 16, 32, 5, HC_LIMITER_MINMOD, 1>(st);
    // 10: 8 warps (30 x 7 tiles), 2 CTAs per SM (128 registers a thread)
    add_march3<10, 8, 32, 5, -1, 2>(st);
    add_march3<10, 8, 32, 5, HC_LIMITER_MINMOD, 2>(st);
    // 11: 14 warps (30 x 13 tiles), 1 CTA per SM (144 registers a thread)
    add_march3<11, 14, 32, 5, -1, 1>(st);
    add_march3<11, 14, 32, 5, HC_LIMITER_MINMOD, 1>(st);
}

}  // namespace fz
}  // namespace hc
