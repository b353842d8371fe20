// hc_plain.cu -- the plain FP64 form: one CUDA kernel per reference kernel.
//
// State is hydro-cl-lua's UBuf: array of cons_t {rho, m.x, m.y, m.z, ETotal,
// ePot} in double, x-fastest, numGhost = 2 ghost layers on each active axis.
// Each kernel covers the same index domain as the reference kernel it stands
// for and evaluates the same expressions in the same order.  This file is
// compiled with -fmad=false so that no multiply-add is contracted: with IEEE
// division and square root, results match a CPU evaluation of the same
// expressions bit for bit.
//
// Reference kernels (paths within hydro-cl-lua):
//   boundary_x/y/z      hydro/solver/gridsolver.lua:638-780, 1070-1213, 1272-1314
//   calcLR ("plm cons") hydro/solver/plm.cl:27-91, 976-997
//   calcFlux            hydro/solver/fvsolver.lua:55-199 -> hydro/flux/roe.cl:17-163
//   calcDerivFromFlux   hydro/solver/fvsolver.cl:6-125
//   multAdd/multAddInto hydro/solver/solverbase.lua:1216-1251
//   constrainU          hydro/eqn/euler.cl:697-717
//   calcDT              hydro/eqn/eqn.lua:1182-1235, hydro/eqn/cl/calcDT.cl:38-73

#include "hc_internal.h"
#include "hc_ref_math.cuh"

#include <cmath>
#include <cstring>
#include <algorithm>
#include <mutex>

namespace hc {

namespace {

constexpr int kGhost = 2;
constexpr int kThreads = 256;

struct Cons { double p[6]; };

using ref::Eos;

__device__ __forceinline__ Eos eosOf(const PlainParams& s) {
    Eos e;
    e.gamma = s.gamma; e.rhoMin = s.rhoMin; e.PMin = s.PMin;
    e.fluxLimiter = s.fluxLimiter; e.slopeLimiter = s.slopeLimiter;
    e.flux = s.flux;
    e.hllcMethod = s.hllcMethod;
    e.recon = s.recon;
    e.entropyFix = s.entropyFix;
    e.entropyFactor = s.entropyFactor;
    return e;
}

__device__ __forceinline__ void cellCoords(const PlainParams& s, long long index, int* i) {
    i[0] = (int)(index % s.gs[0]);
    i[1] = (int)((index / s.gs[0]) % s.gs[1]);
    i[2] = (int)(index / ((long long)s.gs[0] * s.gs[1]));
}
__device__ __forceinline__ bool oob(const PlainParams& s, const int* i, int lhs, int rhs) {
    for (int d = 0; d < s.dim; ++d)
        if (i[d] < lhs || i[d] >= s.gs[d] - rhs) return true;
    return false;
}

// ---- kernels -------------------------------------------------------------

// One thread per line along `side`; the other two axes span their full
// extent (ghosts included), as the generated boundary_<x> kernels do.
__global__ void k_boundary(PlainParams s, Cons* U, int side) {
    int const o1 = (side + 1) % 3, o2 = (side + 2) % 3;
    long long const line = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long const nLines = (long long)s.gs[o1] * s.gs[o2];
    if (line >= nLines) return;
    int c[3];
    c[o1] = (int)(line % s.gs[o1]);
    c[o2] = (int)(line / s.gs[o1]);
    int const gsSide = s.gs[side];
    int const N = gsSide - 2 * kGhost;
    auto at = [&](int j) -> Cons& {
        c[side] = j;
        return U[c[0] + (long long)s.gs[0] * (c[1] + (long long)s.gs[1] * c[2])];
    };
    for (int j = 0; j < kGhost; ++j) {
        for (int mm = 0; mm < 2; ++mm) {
            int const method = s.bc[2 * side + mm];
            int dst, src;
            if (method == HC_BOUNDARY_PERIODIC) {
                if (mm == 0) { dst = j; src = kGhost + (j - kGhost + 2 * N) % N; }
                else { dst = gsSide - 1 - j; src = kGhost + (kGhost - 1 - j) % N; }
            } else if (method == HC_BOUNDARY_MIRROR) {
                if (mm == 0) { dst = j; src = 2 * kGhost - 1 - j; }
                else { dst = gsSide - kGhost + j; src = gsSide - kGhost - 1 - j; }
            } else if (method == HC_BOUNDARY_FREEFLOW) {
                if (mm == 0) { dst = j; src = kGhost; }
                else { dst = gsSide - kGhost + j; src = gsSide - kGhost - 1; }
            } else if (method == HC_BOUNDARY_FIXED) {
                // gridsolver.lua:746-765: the side's constant state (ePot 0)
                Cons& o = at(mm == 0 ? j : gsSide - kGhost + j);
                for (int k = 0; k < 5; ++k) o.p[k] = s.fixedCons[2 * side + mm][k];
                o.p[5] = 0.;
                continue;
            } else if (method == HC_BOUNDARY_LINEAR || method == HC_BOUNDARY_QUADRATIC) {
                // gridsolver.lua:783-858: outward, each ghost from the two
                // (three) cells inside it, all 6 reals
                int d, i1, i2, i3;
                if (mm == 0) { d = kGhost - j - 1; i1 = kGhost - j; i2 = kGhost - j + 1; i3 = kGhost - j + 2; }
                else { d = gsSide - kGhost + j; i1 = gsSide - kGhost + j - 1; i2 = gsSide - kGhost + j - 2; i3 = gsSide - kGhost + j - 3; }
                Cons const a1 = at(i1), a2 = at(i2), a3 = at(i3);
                Cons& o = at(d);
                for (int k = 0; k < 6; ++k)
                    o.p[k] = method == HC_BOUNDARY_LINEAR ? 2. * a1.p[k] - a2.p[k] : 3. * a1.p[k] - 3. * a2.p[k] + a3.p[k];
                continue;
            } else {
                continue;
            }
            Cons const v = at(src);
            Cons& d = at(dst);
            d = v;
            if (method == HC_BOUNDARY_MIRROR) d.p[1 + side] = -1. * d.p[1 + side];
        }
    }
}

__global__ void k_constrainU(PlainParams s, Cons* Ub) {
    long long const index = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (index >= s.numCells) return;
    Eos const e = eosOf(s);
    double U[6];
    for (int j = 0; j < 6; ++j) U[j] = Ub[index].p[j];
    ref::constrain(U, e);
    for (int j = 0; j < 6; ++j) Ub[index].p[j] = U[j];
}

// ULR[2 * (side + dim * index) + {0: L, 1: R}]
__global__ void k_calcLR(PlainParams s, const Cons* Ub, Cons* ULR) {
    long long const index = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (index >= s.numCells) return;
    int i[3];
    cellCoords(s, index, i);
    if (oob(s, i, 1, 1)) return;
    Eos const e = eosOf(s);
    Cons const U = Ub[index];
    for (int side = 0; side < s.dim; ++side) {
        Cons L = U, R = U;
        if (s.recon >= HC_RECON_PLM_CONS) {
            Cons const UL = Ub[index - s.stepsize[side]];
            Cons const UR = Ub[index + s.stepsize[side]];
            ref::plmAny(L.p, R.p, e, UL.p, U.p, UR.p, side);
        }
        ULR[2 * (side + s.dim * index) + 0] = L;
        ULR[2 * (side + s.dim * index) + 1] = R;
    }
}

__global__ void k_calcFlux(PlainParams s, const Cons* Ub, const Cons* ULR, Cons* flux, double dt) {
    long long const index = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (index >= s.numCells) return;
    int i[3];
    cellCoords(s, index, i);
    if (oob(s, i, kGhost, kGhost - 1)) return;
    bool const usePLM = s.recon != HC_RECON_NONE;
    // only the Roe flux takes the flux limiter (fvsolver.lua:62-64)
    bool const lim = s.fluxLimiter > 0 && s.flux == HC_FLUX_ROE;
    for (int side = 0; side < s.dim; ++side) {
        double const dx = s.grid_dx[side];
        long long const indexR = index;
        long long const indexL = index - s.stepsize[side];
        Cons& F = flux[side + s.dim * index];
        double area = 1.;
        for (int k = 0; k < s.dim; ++k) if (k != side) area = area * s.grid_dx[k];
        if (area <= 1e-7) {
            for (int j = 0; j < 6; ++j) F.p[j] = 0;
            continue;
        }
        auto lr = [&](long long iL, long long iR, const double*& a, const double*& b) {
            if (usePLM) {
                a = ULR[2 * (side + s.dim * iL) + 1].p;
                b = ULR[2 * (side + s.dim * iR) + 0].p;
            } else {
                a = Ub[iL].p;
                b = Ub[iR].p;
            }
        };
        const double *UL, *UR, *UL_L = nullptr, *UR_L = nullptr, *UL_R = nullptr, *UR_R = nullptr;
        lr(indexL, indexR, UL, UR);
        double dt_dx = 0.;
        if (lim) {
            dt_dx = dt / dx;
            lr(indexL - s.stepsize[side], indexL, UL_L, UR_L);
            lr(indexR, indexR + s.stepsize[side], UL_R, UR_R);
        }
        Eos const e = eosOf(s);
        if (s.flux == HC_FLUX_RUSANOV) {
            double out[6];
            ref::rusanovFlux(out, e, UL, UR, side);
            for (int j = 0; j < 5; ++j) F.p[j] = out[j];
            continue;
        }
        if (s.flux == HC_FLUX_HLL || s.flux == HC_FLUX_HLLC) {
            // a NaN wave bound assigns nothing: the flux buffer keeps its
            // previous content, as in the reference
            ref::Eig eig;
            ref::eigenForInterface(eig, e, UL, UR);
            double out[6];
            bool const set = s.flux == HC_FLUX_HLL ? ref::hllFlux(out, e, UL, UR, side, eig)
                                                   : ref::hllcFlux(out, e, UL, UR, side, eig);
            if (set)
                for (int j = 0; j < 6; ++j) F.p[j] = out[j];
            continue;
        }
        ref::Iface C, IL, IR;
        ref::makeIface(C, e, UL, UR, side);
        if (lim) {
            ref::makeIface(IL, e, UL_L, UR_L, side);
            ref::makeIface(IR, e, UL_R, UR_R, side);
        }
        double out[6];
        ref::roeFlux(out, e, UL, UR, C, &IL, &IR, side, lim, dt_dx);
        for (int j = 0; j < 6; ++j) F.p[j] = out[j];
    }
}

__global__ void k_calcDerivFromFlux(PlainParams s, const Cons* flux, Cons* deriv) {
    long long const index = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (index >= s.numCells) return;
    int i[3];
    cellCoords(s, index, i);
    if (oob(s, i, kGhost, kGhost)) return;
    double volume = 1.;
    for (int k = 0; k < s.dim; ++k) volume = volume * s.grid_dx[k];
    Cons d = deriv[index];
    for (int side = 0; side < s.dim; ++side) {
        const Cons& fL = flux[side + s.dim * index];
        const Cons& fR = flux[side + s.dim * (index + s.stepsize[side])];
        double areaL = 1.;
        for (int k = 0; k < s.dim; ++k) if (k != side) areaL = areaL * s.grid_dx[k];
        double areaR = areaL;
        if (volume > 1e-7) {
            double const invVolume = 1. / volume;
            if (areaL <= 1e-7) areaL = 0.;
            if (areaR <= 1e-7) areaR = 0.;
            areaL *= invVolume;
            areaR *= invVolume;
            for (int j = 0; j < 5; ++j) d.p[j] -= fR.p[j] * areaR - fL.p[j] * areaL;
        }
    }
    deriv[index] = d;
}

__global__ void k_multAddInto(PlainParams s, Cons* a, const Cons* b, double c) {
    long long const index = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (index >= s.numCells) return;
    int i[3];
    cellCoords(s, index, i);
    if (oob(s, i, kGhost, kGhost)) return;
    for (int j = 0; j < 5; ++j) a[index].p[j] += b[index].p[j] * c;
}

__global__ void k_multAdd(PlainParams s, Cons* a, const Cons* b, const Cons* c, double d) {
    long long const index = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (index >= s.numCells) return;
    int i[3];
    cellCoords(s, index, i);
    if (oob(s, i, kGhost, kGhost)) return;
    for (int j = 0; j < 5; ++j) a[index].p[j] = b[index].p[j] + c[index].p[j] * d;
}

// calcDT cell values folded straight into a per-block minimum: one partial
// per block, reduced again by k_minReduce.  Ghost cells contribute +inf.
__global__ void k_calcDT(PlainParams s, const Cons* Ub, double* partial) {
    long long const index = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double dt = INFINITY;
    if (index < s.numCells) {
        int i[3];
        cellCoords(s, index, i);
        if (!oob(s, i, kGhost, kGhost)) dt = ref::dtCell(Ub[index].p, eosOf(s), s.dim, s.grid_dx);
    }
    for (int o = 16; o > 0; o >>= 1) dt = fmin(dt, __shfl_xor_sync(0xffffffffu, dt, o));
    __shared__ double warpMin[kThreads / 32];
    if ((threadIdx.x & 31) == 0) warpMin[threadIdx.x >> 5] = dt;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = threadIdx.x < blockDim.x / 32 ? warpMin[threadIdx.x] : INFINITY;
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) partial[blockIdx.x] = v;
    }
}

__global__ void k_minReduce(const double* in, long long n, double* out) {
    double v = INFINITY;
    for (long long k = threadIdx.x; k < n; k += blockDim.x) v = fmin(v, in[k]);
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    __shared__ double warpMin[32];
    if ((threadIdx.x & 31) == 0) warpMin[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < blockDim.x / 32 ? warpMin[threadIdx.x] : INFINITY;
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) *out = v;
    }
}

// Kahan-compensated interior sums of the 5 integrated fields times cell
// volume: each block sums its cells with compensation, a single block then
// combines the block sums with compensation in a fixed order.
__global__ void k_sums(PlainParams s, const Cons* Ub, double vol, double* partial) {
    double sum[5] = {0, 0, 0, 0, 0}, comp[5] = {0, 0, 0, 0, 0};
    for (long long index = blockIdx.x * (long long)blockDim.x + threadIdx.x; index < s.numCells;
         index += (long long)gridDim.x * blockDim.x) {
        int i[3];
        cellCoords(s, index, i);
        if (oob(s, i, kGhost, kGhost)) continue;
        for (int j = 0; j < 5; ++j) {
            double const y = Ub[index].p[j] * vol - comp[j];
            double const t = sum[j] + y;
            comp[j] = (t - sum[j]) - y;
            sum[j] = t;
        }
    }
    __shared__ double sh[5][kThreads];
    for (int j = 0; j < 5; ++j) sh[j][threadIdx.x] = sum[j];
    __syncthreads();
    if (threadIdx.x < 5) {
        int const j = threadIdx.x;
        double sm = 0, c = 0;
        for (int k = 0; k < (int)blockDim.x; ++k) {
            double const y = sh[j][k] - c;
            double const t = sm + y;
            c = (t - sm) - y;
            sm = t;
        }
        partial[5 * blockIdx.x + j] = sm;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct PlainSolver {
    PlainParams p;
    cudaStream_t stream;
    Cons* U = nullptr;
    Cons* ULR = nullptr;
    Cons* flux = nullptr;
    Cons* UBufs[4] = {nullptr, nullptr, nullptr, nullptr};
    Cons* derivs[4] = {nullptr, nullptr, nullptr, nullptr};
    double* partial = nullptr;   // calcDT / sums scratch
    double* scalar = nullptr;
    double* host_scalar = nullptr;
    void* staging = nullptr;     // device staging for layout conversion
    int order = 1;
    long long blocks = 0;
};

long long plain_num_cells(const PlainSolver* p) { return p->p.numCells; }
const double* plain_state_dev(const PlainSolver* p) { return reinterpret_cast<const double*>(p->U); }

static int alloc(void** ptr, size_t bytes) {
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc");
    return HC_OK;
}

int plain_create(const hc_solver_desc& d, cudaStream_t stream, PlainSolver** out) {
    PlainSolver* s = new PlainSolver();
    PlainParams& p = s->p;
    p.dim = d.dim;
    for (int k = 0; k < 3; ++k) {
        int const n = k < d.dim ? d.n[k] : 1;
        p.gs[k] = k < d.dim ? n + 2 * kGhost : 1;
        p.grid_dx[k] = (d.maxs[k] - d.mins[k]) / (double)n;
    }
    p.stepsize[0] = 1;
    p.stepsize[1] = p.gs[0];
    p.stepsize[2] = p.gs[0] * p.gs[1];
    p.numCells = (long long)p.gs[0] * p.gs[1] * p.gs[2];
    for (int k = 0; k < 6; ++k) p.bc[k] = d.boundary[k];
    p.fluxLimiter = d.flux_limiter;
    p.recon = d.recon;
    p.slopeLimiter = d.slope_limiter;
    p.flux = d.flux;
    p.hllcMethod = d.hllc_method == HC_HLLC_DEFAULT ? 2 : d.hllc_method - 1;
    p.gamma = d.gamma;
    p.rhoMin = d.rho_min;
    p.PMin = d.p_min;
    p.entropyFix = d.entropy_fix != 0;
    p.entropyFactor = d.entropy_fix_factor;
    std::memcpy(p.fixedCons, d.fixed_cons, sizeof(p.fixedCons));
    s->stream = stream;
    s->order = rk_table(d.integrator).order;
    s->blocks = (p.numCells + kThreads - 1) / kThreads;
    size_t const nc = (size_t)p.numCells;
    int r = HC_OK;
    if (r == HC_OK) r = alloc((void**)&s->U, nc * sizeof(Cons));
    if (r == HC_OK && d.recon != HC_RECON_NONE) r = alloc((void**)&s->ULR, 2 * nc * d.dim * sizeof(Cons));
    if (r == HC_OK) r = alloc((void**)&s->flux, nc * d.dim * sizeof(Cons));
    for (int k = 0; k < s->order && r == HC_OK; ++k) {
        r = alloc((void**)&s->derivs[k], nc * sizeof(Cons));
        if (r == HC_OK && d.integrator != HC_INT_FORWARD_EULER) r = alloc((void**)&s->UBufs[k], nc * sizeof(Cons));
    }
    if (r == HC_OK) r = alloc((void**)&s->partial, std::max<long long>(s->blocks, 5 * 1024) * sizeof(double));
    if (r == HC_OK) r = alloc((void**)&s->scalar, 8 * sizeof(double));
    if (r == HC_OK) r = alloc(&s->staging, nc * 6 * sizeof(double));
    if (r == HC_OK) {
        cudaError_t e = cudaMallocHost((void**)&s->host_scalar, 8 * sizeof(double));
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMallocHost");
    }
    if (r == HC_OK) {
        cudaError_t e = cudaMemsetAsync(s->U, 0, nc * sizeof(Cons), stream);
        if (e == cudaSuccess && s->flux) e = cudaMemsetAsync(s->flux, 0, nc * d.dim * sizeof(Cons), stream);
        if (e == cudaSuccess && s->ULR) e = cudaMemsetAsync(s->ULR, 0, 2 * nc * d.dim * sizeof(Cons), stream);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMemsetAsync");
    }
    if (r != HC_OK) {
        plain_destroy(s);
        return r;
    }
    *out = s;
    return HC_OK;
}

void plain_destroy(PlainSolver* s) {
    if (!s) return;
    cudaFree(s->U);
    cudaFree(s->ULR);
    cudaFree(s->flux);
    for (int k = 0; k < 4; ++k) { cudaFree(s->UBufs[k]); cudaFree(s->derivs[k]); }
    cudaFree(s->partial);
    cudaFree(s->scalar);
    cudaFree(s->staging);
    if (s->host_scalar) cudaFreeHost(s->host_scalar);
    delete s;
}

int plain_set_full(PlainSolver* s, const double* host) {
    HC_CUDA(cudaMemcpyAsync(s->U, host, s->p.numCells * sizeof(Cons), cudaMemcpyHostToDevice, s->stream));
    HC_CUDA(cudaStreamSynchronize(s->stream));
    return HC_OK;
}

int plain_get_full(PlainSolver* s, double* host) {
    HC_CUDA(cudaMemcpyAsync(host, s->U, s->p.numCells * sizeof(Cons), cudaMemcpyDeviceToHost, s->stream));
    HC_CUDA(cudaStreamSynchronize(s->stream));
    return HC_OK;
}

namespace {
// Interior <-> full-grid scatter/gather with layout conversion.
// layout: 0 = AoS6 f64, 1 = SoA5 f64, 2 = SoA5 f32.  dir 0: host -> grid.
__global__ void k_interior_xfer(PlainParams s, Cons* U, void* host, int layout, int dir) {
    long long const nx = s.gs[0] - (s.dim > 0 ? 2 * kGhost : 0);
    long long const ny = s.dim > 1 ? s.gs[1] - 2 * kGhost : 1;
    long long const nz = s.dim > 2 ? s.gs[2] - 2 * kGhost : 1;
    long long const n = nx * ny * nz;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        long long const x = k % nx, y = (k / nx) % ny, z = k / (nx * ny);
        long long const gx = x + kGhost, gy = y + (s.dim > 1 ? kGhost : 0), gz = z + (s.dim > 2 ? kGhost : 0);
        Cons& c = U[gx + s.gs[0] * (gy + (long long)s.gs[1] * gz)];
        for (int j = 0; j < 6; ++j) {
            if (layout != 0 && j == 5) {
                if (dir == 0) c.p[5] = 0.;
                continue;
            }
            if (layout == 0) {
                double* h = (double*)host + 6 * k + j;
                if (dir == 0) c.p[j] = *h; else *h = c.p[j];
            } else if (layout == 1) {
                double* h = (double*)host + j * n + k;
                if (dir == 0) c.p[j] = *h; else *h = c.p[j];
            } else {
                float* h = (float*)host + j * n + k;
                if (dir == 0) c.p[j] = (double)*h; else *h = (float)c.p[j];
            }
        }
    }
}

size_t layout_bytes(long long n, int layout) {
    return layout == HC_LAYOUT_AOS6_F64 ? n * 6 * sizeof(double)
         : layout == HC_LAYOUT_SOA5_F64 ? n * 5 * sizeof(double) : n * 5 * sizeof(float);
}

long long interior_count(const PlainParams& s) {
    long long n = 1;
    for (int d = 0; d < s.dim; ++d) n *= s.gs[d] - 2 * kGhost;
    return n;
}
}  // namespace

int plain_set_interior(PlainSolver* s, const void* host, int layout) {
    long long const n = interior_count(s->p);
    HC_CUDA(cudaMemcpyAsync(s->staging, host, layout_bytes(n, layout), cudaMemcpyHostToDevice, s->stream));
    k_interior_xfer<<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256, 0, s->stream>>>(s->p, s->U, s->staging, layout, 0);
    HC_CUDA(cudaGetLastError());
    HC_CUDA(cudaStreamSynchronize(s->stream));
    return HC_OK;
}

// The reference's UBuf (AoS-6, ghosts included) of a solver described by d,
// from its interior cells in device memory: the interior is placed and the
// ghosts filled by the plain form's boundary kernels (gridsolver.lua:638-780,
// x then y then z, corners included).  Used to export the state of the fused
// forms, which keep no corner ghosts, in the reference's layout.
int plain_expand_full(const hc_solver_desc& d, const void* interior_dev, int layout, double* full_dev, cudaStream_t stream) {
    PlainParams p;
    std::memset(&p, 0, sizeof(p));
    p.dim = d.dim;
    for (int k = 0; k < 3; ++k) {
        int const n = k < d.dim ? d.n[k] : 1;
        p.gs[k] = k < d.dim ? n + 2 * kGhost : 1;
        p.grid_dx[k] = (d.maxs[k] - d.mins[k]) / (double)n;
    }
    p.stepsize[0] = 1;
    p.stepsize[1] = p.gs[0];
    p.stepsize[2] = p.gs[0] * p.gs[1];
    p.numCells = (long long)p.gs[0] * p.gs[1] * p.gs[2];
    for (int k = 0; k < 6; ++k) p.bc[k] = d.boundary[k];
    std::memcpy(p.fixedCons, d.fixed_cons, sizeof(p.fixedCons));
    p.gamma = d.gamma;
    p.rhoMin = d.rho_min;
    p.PMin = d.p_min;
    long long const n = interior_count(p);
    HC_CUDA(cudaMemsetAsync(full_dev, 0, (size_t)p.numCells * sizeof(Cons), stream));
    k_interior_xfer<<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256, 0, stream>>>(
        p, reinterpret_cast<Cons*>(full_dev), const_cast<void*>(interior_dev), layout, 0);
    for (int side = 0; side < p.dim; ++side) {
        int const o1 = (side + 1) % 3, o2 = (side + 2) % 3;
        long long const lines = (long long)p.gs[o1] * p.gs[o2];
        k_boundary<<<(unsigned)((lines + 127) / 128), 128, 0, stream>>>(p, reinterpret_cast<Cons*>(full_dev), side);
    }
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int plain_init_state(PlainSolver* s, const hc_init& ic, const hc_solver_desc& d) {
    long long const n = interior_count(s->p);
    HC_CHECK(init_fill(ic, d, static_cast<double*>(s->staging), s->stream));
    k_interior_xfer<<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256, 0, s->stream>>>(
        s->p, s->U, s->staging, HC_LAYOUT_AOS6_F64, 0);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int plain_get_interior(PlainSolver* s, void* host, int layout) {
    long long const n = interior_count(s->p);
    k_interior_xfer<<<(unsigned)std::min<long long>((n + 255) / 256, 4096), 256, 0, s->stream>>>(s->p, s->U, s->staging, layout, 1);
    HC_CUDA(cudaGetLastError());
    HC_CUDA(cudaMemcpyAsync(host, s->staging, layout_bytes(n, layout), cudaMemcpyDeviceToHost, s->stream));
    HC_CUDA(cudaStreamSynchronize(s->stream));
    return HC_OK;
}

static int launch_boundary(PlainSolver* s, Cons* U) {
    for (int side = 0; side < s->p.dim; ++side) {
        int const o1 = (side + 1) % 3, o2 = (side + 2) % 3;
        long long const lines = (long long)s->p.gs[o1] * s->p.gs[o2];
        k_boundary<<<(unsigned)((lines + 127) / 128), 128, 0, s->stream>>>(s->p, U, side);
    }
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int plain_boundary(PlainSolver* s) { return launch_boundary(s, s->U); }

int plain_constrain_u(PlainSolver* s) {
    k_constrainU<<<(unsigned)s->blocks, kThreads, 0, s->stream>>>(s->p, s->U);
    HC_CUDA(cudaGetLastError());
    return launch_boundary(s, s->U);
}

int plain_calc_dt(PlainSolver* s, double cfl, double fixed_dt, double* dt) {
    if (fixed_dt > 0) { *dt = fixed_dt; return HC_OK; }
    k_calcDT<<<(unsigned)s->blocks, kThreads, 0, s->stream>>>(s->p, s->U, s->partial);
    k_minReduce<<<1, 1024, 0, s->stream>>>(s->partial, s->blocks, s->scalar);
    HC_CUDA(cudaGetLastError());
    HC_CUDA(cudaMemcpyAsync(s->host_scalar, s->scalar, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    HC_CUDA(cudaStreamSynchronize(s->stream));
    *dt = cfl * s->host_scalar[0];
    return HC_OK;
}

static int calc_deriv(PlainSolver* s, Cons* deriv, double dt) {
    unsigned const g = (unsigned)s->blocks;
    if (s->p.recon != HC_RECON_NONE) k_calcLR<<<g, kThreads, 0, s->stream>>>(s->p, s->U, s->ULR);
    k_calcFlux<<<g, kThreads, 0, s->stream>>>(s->p, s->U, s->ULR, s->flux, dt);
    k_calcDerivFromFlux<<<g, kThreads, 0, s->stream>>>(s->p, s->flux, deriv);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

// hydro/int/fe.lua:33-49 and hydro/int/rk.lua:98-218
int plain_step(PlainSolver* s, int integrator, double dt) {
    size_t const bytes = (size_t)s->p.numCells * sizeof(Cons);
    unsigned const g = (unsigned)s->blocks;
    if (integrator == HC_INT_FORWARD_EULER) {
        HC_CUDA(cudaMemsetAsync(s->derivs[0], 0, bytes, s->stream));
        HC_CHECK(calc_deriv(s, s->derivs[0], dt));
        k_multAddInto<<<g, kThreads, 0, s->stream>>>(s->p, s->U, s->derivs[0], dt);
        HC_CHECK(launch_boundary(s, s->U));
        return plain_constrain_u(s);
    }
    const RKTable& T = rk_table(integrator);
    int const order = T.order;
    auto alphaNeeded = [&](int i) { for (int m = i; m <= order; ++m) if (T.alpha[m - 1][i - 1] != 0) return true; return false; };
    auto betaNeeded = [&](int i) { for (int m = i; m <= order; ++m) if (T.beta[m - 1][i - 1] != 0) return true; return false; };
    if (alphaNeeded(1)) HC_CUDA(cudaMemcpyAsync(s->UBufs[0], s->U, bytes, cudaMemcpyDeviceToDevice, s->stream));
    if (betaNeeded(1)) {
        HC_CUDA(cudaMemsetAsync(s->derivs[0], 0, bytes, s->stream));
        HC_CHECK(calc_deriv(s, s->derivs[0], dt));
    }
    for (int i = 2; i <= order + 1; ++i) {
        HC_CUDA(cudaMemsetAsync(s->U, 0, bytes, s->stream));
        for (int k = 1; k <= i - 1; ++k)
            if (T.alpha[i - 2][k - 1] != 0)
                k_multAdd<<<g, kThreads, 0, s->stream>>>(s->p, s->U, s->U, s->UBufs[k - 1], T.alpha[i - 2][k - 1]);
        for (int k = 1; k <= i - 1; ++k)
            if (T.beta[i - 2][k - 1] != 0)
                k_multAdd<<<g, kThreads, 0, s->stream>>>(s->p, s->U, s->U, s->derivs[k - 1], T.beta[i - 2][k - 1] * dt);
        HC_CUDA(cudaGetLastError());
        HC_CHECK(launch_boundary(s, s->U));
        HC_CHECK(plain_constrain_u(s));
        if (i <= order) {
            if (alphaNeeded(i)) HC_CUDA(cudaMemcpyAsync(s->UBufs[i - 1], s->U, bytes, cudaMemcpyDeviceToDevice, s->stream));
            if (betaNeeded(i)) {
                HC_CUDA(cudaMemsetAsync(s->derivs[i - 1], 0, bytes, s->stream));
                HC_CHECK(calc_deriv(s, s->derivs[i - 1], dt));
            }
        }
    }
    return HC_OK;
}

int plain_conservation(PlainSolver* s, double sums[5]) {
    double vol = 1.;
    for (int k = 0; k < s->p.dim; ++k) vol *= s->p.grid_dx[k];
    int const blocks = 1024;
    k_sums<<<blocks, kThreads, 0, s->stream>>>(s->p, s->U, vol, s->partial);
    HC_CUDA(cudaGetLastError());
    std::vector<double> part(5 * blocks);
    HC_CUDA(cudaMemcpyAsync(part.data(), s->partial, part.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    HC_CUDA(cudaStreamSynchronize(s->stream));
    for (int j = 0; j < 5; ++j) {
        double sm = 0, c = 0;
        for (int b = 0; b < blocks; ++b) {
            double const y = part[5 * b + j] - c;
            double const t = sm + y;
            c = (t - sm) - y;
            sm = t;
        }
        sums[j] = sm;
    }
    return HC_OK;
}

}  // namespace hc

// ---------------------------------------------------------------------------
// calcDT without allocation
//
// For callers that cannot allocate device memory at the moment they need a
// time step: code that is recording a CUDA graph (cudaMalloc is not a stream
// operation and is refused during stream capture), code that runs under an
// external memory manager that owns every byte of the device, or a real-time
// loop that cannot afford the implicit device synchronisation of cudaMalloc.
// They pass the state and the output in memory they already own; the
// per-block minima of the reduction live in this fixed array inside the
// library instead of in a scratch buffer.
// ---------------------------------------------------------------------------

namespace hc {
namespace {

constexpr long long kNoAllocBlocks = HC_NOALLOC_MAX_CELLS / kThreads;

// Block minima of k_calcDT.  Every device that loads the library holds this
// array (512 KiB) until the process exits.  All calls share it: each call
// writes entries [0, blocks) before reading them, so nothing has to start at
// zero, but two calls whose kernels overlap on the GPU race on it.
static __device__ __align__(256) double g_noalloc_partial[kNoAllocBlocks];

// cfl * min over the block minima (or the fixed dt), written to device memory
__global__ void k_minReduceScaled(const double* in, long long n, double cfl, double* out) {
    double v = INFINITY;
    for (long long k = threadIdx.x; k < n; k += blockDim.x) v = fmin(v, in[k]);
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    __shared__ double warpMin[32];
    if ((threadIdx.x & 31) == 0) warpMin[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < blockDim.x / 32 ? warpMin[threadIdx.x] : INFINITY;
        for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (threadIdx.x == 0) *out = cfl * v;
    }
}

__global__ void k_writeScalar(double v, double* out) { *out = v; }

// Device address of g_noalloc_partial per device, looked up once per device
// (with that device current) on its first call and kept for the life of the
// process: after a cudaDeviceReset the module may load elsewhere, so the entry
// point is not for use after one (see the header).
constexpr int kMaxDevices = 64;
double* g_noalloc_ptr[kMaxDevices] = {nullptr};
std::mutex g_noalloc_mutex;

int noalloc_scratch(double** out) {
    int dev = 0;
    HC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(HC_ERR_INVALID, "device index beyond the supported range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partial);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_partial)");
        g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return HC_OK;
}

}  // namespace

}  // namespace hc

extern "C" int hc_calc_dt_noalloc(const hc_solver_desc* d, const double* state, double* dt_out, void* stream) {
    using namespace hc;
    if (!d || !state || !dt_out) return fail(HC_ERR_INVALID, "NULL argument");
    // the fields this call reads, with the rules hc_solver_create applies
    if (d->dim < 1 || d->dim > 3) return fail(HC_ERR_INVALID, "dim must be 1, 2 or 3");
    for (int k = 0; k < d->dim; ++k) {
        if (d->n[k] < 2) return fail(HC_ERR_INVALID, "each active axis needs at least 2 cells");
        if (d->n[k] > HC_NOALLOC_MAX_CELLS)
            return fail(HC_ERR_INVALID, "hc_calc_dt_noalloc: the grid has more than HC_NOALLOC_MAX_CELLS cells");
        if (!(d->maxs[k] > d->mins[k])) return fail(HC_ERR_INVALID, "maxs must exceed mins");
    }
    if (!(d->gamma > 1.)) return fail(HC_ERR_INVALID, "gamma must exceed 1");
    if (!(d->cfl > 0.) && !(d->fixed_dt > 0.)) return fail(HC_ERR_INVALID, "cfl or fixed_dt must be positive");
    PlainParams p;
    std::memset(&p, 0, sizeof(p));
    p.dim = d->dim;
    long long cells = 1;
    for (int k = 0; k < 3; ++k) {
        int const n = k < d->dim ? d->n[k] : 1;
        p.gs[k] = k < d->dim ? n + 2 * kGhost : 1;
        p.grid_dx[k] = (d->maxs[k] - d->mins[k]) / (double)n;
        cells *= p.gs[k];
        if (cells > HC_NOALLOC_MAX_CELLS)
            return fail(HC_ERR_INVALID, "hc_calc_dt_noalloc: the grid (ghosts included) has more than HC_NOALLOC_MAX_CELLS cells");
    }
    p.stepsize[0] = 1;
    p.stepsize[1] = p.gs[0];
    p.stepsize[2] = p.gs[0] * p.gs[1];
    p.numCells = cells;
    p.gamma = d->gamma;
    p.rhoMin = d->rho_min;
    p.PMin = d->p_min;
    // the per-device set-up (the scratch array's address) happens on every
    // first call on a device, whatever the descriptor asks for
    double* scratch = nullptr;
    HC_CHECK(noalloc_scratch(&scratch));
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    if (d->fixed_dt > 0) {
        k_writeScalar<<<1, 1, 0, s>>>(d->fixed_dt, dt_out);
        HC_CUDA(cudaGetLastError());
        return HC_OK;
    }
    long long const blocks = (p.numCells + kThreads - 1) / kThreads;
    k_calcDT<<<(unsigned)blocks, kThreads, 0, s>>>(p, reinterpret_cast<const Cons*>(state), scratch);
    k_minReduceScaled<<<1, 1024, 0, s>>>(scratch, blocks, d->cfl, dt_out);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}
