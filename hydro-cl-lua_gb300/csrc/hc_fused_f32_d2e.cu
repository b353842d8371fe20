// hc_fused_f32_d2e.cu -- 2D stage kernels, FP32 (fast form): 8-cell segments
// with the sliding window unrolled by 2 (the rotation of the window's
// registers then needs no copies) at 128 registers a thread, on smaller tiles
// (less padding in the partial tiles at grid edges, more CTAs per SM) and on
// the transposed 32x64 tile.  (32x16 and 16x32 tiles at 64 threads and 8 CTAs
// per SM measured 4-5 % slower than 32x32 at 128 threads: their halo is 1.41x
// the interior against 1.27x.  The 32x32 tile with the window not unrolled
// measured 2.5 % slower, with the epilogue's cell loop unrolled by 2 18 %
// slower, at 3 CTAs per SM (166 registers) 16 % slower.)
#include "hc_fused_inst.cuh"

namespace hc {
namespace fz {

void register_f32_d2e(std::vector<StageLauncher>& st, std::vector<AuxLauncher>& aux) {
    using T = float;
    constexpr int P = HC_F32_FUSED;
    (void)aux;
    // 10: 32x32, 128 threads, 4 CTAs per SM
    // 11: 64x16, 128 threads, 4 CTAs per SM
    // 12: 32x64, 256 threads, 2 CTAs per SM
    add_plm_set<T, P, 2, 10, 32, 32, 1, 8, 128, 2, 4>(st);   // every compiled-in limiter
    add_plm_pair<T, P, 2, 11, 64, 16, 1, 8, 128, 2, 4>(st);
    add_plm_pair<T, P, 2, 12, 32, 64, 1, 8, 256, 2, 2>(st);
}

}  // namespace fz
}  // namespace hc
