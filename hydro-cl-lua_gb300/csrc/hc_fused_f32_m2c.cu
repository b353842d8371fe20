// hc_fused_f32_m2c.cu -- the 2D marching kernel of schedule 17 (3 CTAs per
// SM) with segments of 128 rows: half the rows a segment loads and primes
// beside its own on the large batched grids.
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_m2c(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    (void)aux;
    add_march2<21, 4, 128, 8, 2, -1, 3>(st);
    add_march2<21, 4, 128, 8, 2, HC_LIMITER_VAN_LEER_ABS, 3>(st);
    add_march2<21, 4, 128, 8, 2, HC_LIMITER_MONOTIZED_CENTRAL, 3>(st);
    add_march2<21, 4, 128, 8, 2, HC_LIMITER_MINMOD, 3>(st);
}

}  // namespace fz
}  // namespace hc
