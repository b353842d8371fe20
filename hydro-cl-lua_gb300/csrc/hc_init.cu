// hc_init.cu -- initial conditions generated on the device.
//
// hydro-cl-lua builds every initial state with a kernel (the initCond's
// applyInitCond, hydro/solver/solverbase.lua:2094-2136, gridsolver.lua:530-544)
// rather than on the host.  This file does the same for the states the
// configurations use, so a solve can be admitted without building and
// uploading its state from the host: the kernel writes the interior cells in
// the AoS-6 FP64 layout (x fastest) into device memory, and the caller feeds
// that buffer to the same transfer kernel a host upload goes through.
//
// Every value is computed in double with the expressions, in the order, of
// the host generators (hydrocuda.py: cell_centers, cons_from_prim, sod_state,
// blast_state, quadrant_state, kelvin_helmholtz_state), compiled without FMA
// contraction, so a device-initialised solve is bit-identical to one admitted
// from the host generator's array.
//   Sod            hydro/init/euler.lua:742-752 (left where x < mid on every active axis)
//   blast          rho = 1, v = 0, P = Pin inside |x| < radius, Pout outside
//   quadrant       hydro/init/euler.lua:249-283 (quadrant order (+,+), (-,+), (-,-), (+,-))
//   Kelvin-Helmholtz  the sharp-band form: |y| < 0.25 has rho = 2, vx = .5, else
//                  rho = 1, vx = -.5; P = 2.5; vy = noise * U(-1, 1) from
//                  SplitMix64(seed), one draw per cell in x-fastest order
#include "hc_internal.h"

#include <cstring>

namespace hc {
namespace {

__device__ __forceinline__ double cellCenter(int i, int n, double lo, double hi) {
    // (i + G + .5 - G) / N * (max - min) + min with G = 2 (coord.lua:1399-1440)
    double const ig = (double)(i + 2);
    return (ig + .5 - 2.) / (double)n * (hi - lo) + lo;
}

// The k-th (0-based) uniform in [0, 1) of SplitMix64(seed).
__device__ __forceinline__ double splitmixUniform(unsigned long long seed, unsigned long long k) {
    unsigned long long z = seed + (k + 1ull) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

struct InitArgs {
    hc_init ic;
    int dim, n[3];
    double mins[3], maxs[3], gamma;
};

__global__ void k_init(InitArgs a, double* out) {
    long long const nx = a.n[0], ny = a.n[1], nz = a.n[2];
    long long const total = nx * ny * nz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
         c += (long long)gridDim.x * blockDim.x) {
        int const i = (int)(c % nx), j = (int)((c / nx) % ny), k = (int)(c / (nx * ny));
        double X[3] = {0., 0., 0.};
        int const idx[3] = {i, j, k};
        for (int d = 0; d < a.dim; ++d) X[d] = cellCenter(idx[d], a.n[d], a.mins[d], a.maxs[d]);
        double rho = 1., vx = 0., vy = 0., vz = 0., P = 1.;
        const double* p = a.ic.p;
        switch (a.ic.kind) {
        case HC_INIT_SOD: {
            bool left = true;
            for (int d = 0; d < a.dim; ++d) left = left && X[d] < (a.mins[d] + a.maxs[d]) * .5;
            rho = left ? p[0] : p[2];
            P = left ? p[1] : p[3];
            break;
        }
        case HC_INIT_BLAST: {
            double r2 = 0.;
            for (int d = 0; d < a.dim; ++d) r2 = r2 + X[d] * X[d];
            P = r2 < p[0] * p[0] ? p[1] : p[2];
            rho = p[3];
            break;
        }
        case HC_INIT_QUADRANT: {
            bool const xp = X[0] > (a.mins[0] + a.maxs[0]) * .5;
            bool const yp = X[1] > (a.mins[1] + a.maxs[1]) * .5;
            int const q = yp ? (xp ? 0 : 1) : (!xp ? 2 : 3);
            rho = p[4 * q + 0];
            vx = p[4 * q + 1];
            vy = p[4 * q + 2];
            P = p[4 * q + 3];
            break;
        }
        default: {   // HC_INIT_KELVIN_HELMHOLTZ
            bool const inside = fabs(X[1]) < 0.25;
            rho = inside ? 2.0 : 1.0;
            vx = inside ? 0.5 : -0.5;
            vy = p[0] * (-1.0 + (1.0 - -1.0) * splitmixUniform(a.ic.seed, (unsigned long long)c));
            P = 2.5;
            break;
        }
        }
        double* o = out + 6 * c;
        o[0] = rho;
        o[1] = vx * rho;
        o[2] = vy * rho;
        o[3] = vz * rho;
        o[4] = rho * (.5 * (vx * vx + vy * vy + vz * vz)) + P / (a.gamma - 1.);
        o[5] = 0.;
    }
}

}  // namespace

int init_validate(const hc_init& ic, const hc_solver_desc& d) {
    if (ic.kind < 0 || ic.kind > HC_INIT_KELVIN_HELMHOLTZ) return fail(HC_ERR_INVALID, "unknown initial condition");
    if ((ic.kind == HC_INIT_QUADRANT || ic.kind == HC_INIT_KELVIN_HELMHOLTZ) && d.dim != 2)
        return fail(HC_ERR_INVALID, "the quadrant and Kelvin-Helmholtz initial conditions are two-dimensional");
    return HC_OK;
}

int init_fill(const hc_init& ic, const hc_solver_desc& d, double* dst, cudaStream_t s) {
    HC_CHECK(init_validate(ic, d));
    InitArgs a;
    a.ic = ic;
    a.dim = d.dim;
    long long total = 1;
    for (int k = 0; k < 3; ++k) {
        a.n[k] = k < d.dim ? d.n[k] : 1;
        a.mins[k] = d.mins[k];
        a.maxs[k] = d.maxs[k];
        total *= a.n[k];
    }
    a.gamma = d.gamma;
    long long const blocks = (total + 255) / 256;
    k_init<<<(unsigned)(blocks < 4096 ? (blocks < 1 ? 1 : blocks) : 4096), 256, 0, s>>>(a, dst);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

}  // namespace hc

extern "C" int hc_init_defaults(int kind, hc_init* out) {
    using namespace hc;
    if (!out) return fail(HC_ERR_INVALID, "out is NULL");
    hc_init z;
    std::memset(&z, 0, sizeof(z));
    z.kind = kind;
    switch (kind) {
    case HC_INIT_SOD: z.p[0] = 1.; z.p[1] = 1.; z.p[2] = .125; z.p[3] = .1; break;
    case HC_INIT_BLAST: z.p[0] = .2; z.p[1] = 1.; z.p[2] = .1; z.p[3] = 1.; break;
    case HC_INIT_QUADRANT: {
        // 'configuration 1' of the reference's quadrant problems (hydro/init/euler.lua:1516-1522),
        // as (rho, vx, vy, P) per quadrant
        double const q[16] = {1., 0., 0., 1., .5197, -.7259, 0., .4, .1072, -.7259, -1.4045, .0439,
                              .2579, 0., -1.4045, .15};
        for (int k = 0; k < 16; ++k) z.p[k] = q[k];
        break;
    }
    case HC_INIT_KELVIN_HELMHOLTZ: z.p[0] = .01; z.seed = 2; break;
    default: return fail(HC_ERR_INVALID, "unknown initial condition");
    }
    *out = z;
    return HC_OK;
}
