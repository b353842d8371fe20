// hc_fused_f32_recon.cu -- FP32 stage kernels (fast form) for the Roe flux with
// "plm prim" or "plm athena" (hydro/solver/plm.cl:191-253, 782-879): one
// schedule per dimension, the reconstruction kind and the slope limiter read
// from the scheme at run time.  ("plm cons" has its own tuned schedules.)
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_recon(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    (void)aux;
    using T = float;
    constexpr int P = HC_F32_FUSED;
    constexpr bool E = false;
    // compiled for 128 registers a thread (16 and 2 CTAs per SM in 1D and
    // 2D): the athena reconstruction spills at 64
    add_stage<T, P, 1, 0, 128, 1, 1, 4, 32, E, -1, false, -1, 0, 16>(st);
    add_stage<T, P, 2, 0, 32, 32, 1, 4, 256, E, -1, false, -1, 0, 2>(st);
    add_stage<T, P, 3, 0, 16, 8, 8, 4, 256, E, -1, false>(st);
}

}  // namespace fz
}  // namespace hc
