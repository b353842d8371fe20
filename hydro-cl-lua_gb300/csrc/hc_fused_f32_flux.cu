// hc_fused_f32_flux.cu -- FP32 stage kernels (fast form) for the HLL, Rusanov
// and HLLC interface fluxes (hydro/flux/hll.cl, rusanov.cl, euler-hllc.cl): one
// schedule per dimension, with any PLM reconstruction (the kind and the slope
// limiter chosen at run time) and without.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

template <int FLUX>
static void add_flux_kernels(std::vector<StageLauncher>& st) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    constexpr bool E = false;
    // the PLM kernels are compiled for 128 registers a thread (16 and 2 CTAs
    // per SM in 1D and 2D): the athena reconstruction spills at 64
    add_stage<T, P, 1, 0, 128, 1, 1, 4, 32, E, -1, false, -1, 0, 16, 1, FLUX>(st);
    add_stage<T, P, 1, 0, 128, 1, 1, 4, 32, E, 0, false, -1, 0, 0, 1, FLUX>(st);
    add_stage<T, P, 2, 0, 32, 32, 1, 4, 256, E, -1, false, -1, 0, 2, 1, FLUX>(st);
    add_stage<T, P, 2, 0, 32, 32, 1, 4, 256, E, 0, false, -1, 0, 0, 1, FLUX>(st);
    add_stage<T, P, 3, 0, 16, 8, 8, 4, 256, E, -1, false, -1, 0, 0, 1, FLUX>(st);
    add_stage<T, P, 3, 0, 16, 8, 8, 4, 256, E, 0, false, -1, 0, 0, 1, FLUX>(st);
}

void register_f32_flux(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    (void)aux;
    add_flux_kernels<HC_FLUX_HLL>(st);
    add_flux_kernels<HC_FLUX_RUSANOV>(st);
    add_flux_kernels<HC_FLUX_HLLC>(st);
}

}  // namespace fz
}  // namespace hc
