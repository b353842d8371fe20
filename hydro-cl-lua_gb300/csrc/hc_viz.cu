// hc_viz.cu -- headless visualisation: the reference's display variables,
// their range, mean and deviation, and the arithmetic of its heat-map,
// volume and line-integral-convolution shaders, as CUDA kernels writing
// device buffers (no graphics API is involved).
//
//   display variables    hydro/eqn/euler.lua:240-260 (+ the state fields,
//                        hydro/eqn/eqn.lua:913-915), hydro/eqn/euler.cl:1-112
//   calcDisplayVarToBuffer  hydro/solver/solverbase.lua:1950-2065: every cell
//                        of the grid, ghosts included; a ghost cell shows the
//                        nearest interior cell, or 0 with zeroBorder
//   range / mean / dev.  hydro/solver/solverbase.lua:2871-2994
//   palette              hydro/draw/palette.lua, hydro/app.lua:1229-1241,
//                        hydro/draw/draw.glsl:43-85
//   heat map             hydro/draw/2d_heatmap.glsl:28-59
//   volume ray march     hydro/draw/volumetric.glsl:45-110
//   LIC                  hydro/draw/vector_lic.glsl:36-107, vector_lic.lua
//   slice stack          hydro/draw/3d_slice.glsl:56-118, 3d_slice.lua:165-235
//
// The display values are computed in double with the reference's
// expressions (this file is compiled without FMA contraction).  The image
// kernels compute in float, as the shaders do; textures are sampled the way
// the reference's are set up (GL_LINEAR magnification, GL_REPEAT wrap).
#include "hc_internal.h"

#include <cmath>
#include <initializer_list>
#include <cstring>
#include <vector>

namespace hc {
namespace viz {

// ---- display variables --------------------------------------------------------

// The state on the device: AoS-6 FP64 interior cells; `stride` is the cell
// distance between neighbours along each axis.
struct Grid {
    const double* U;
    long long stride[3];
    int dim, n[3];
    double mins[3], maxs[3];
    double gamma, rhoMin, PMin;
};

// hydro/materials.lua:61 (Air.C_v, J / (kg K)) for calc_T
constexpr double kAirCv = 717.1;

__device__ __forceinline__ double lenSq3(double x, double y, double z) { return x * x + y * y + z * z; }

__device__ double displayValue(const Grid& g, const double* U, int var) {
    // primFromCons (euler.cl:140-159): its guarded branch is overwritten
    double const rho = U[0];
    double const inv = 1. / rho;
    double const vx = U[1] * inv, vy = U[2] * inv, vz = U[3] * inv;
    double const EKinC = U[0] < g.rhoMin ? 0. : (.5 * lenSq3(U[1], U[2], U[3]) / U[0]);
    double const P = U[0] < g.rhoMin ? 0. : ((g.gamma - 1.) * (U[4] - EKinC));
    auto Cs = [&]() -> double {
        if (P <= g.PMin) return 0.;
        if (rho < g.rhoMin) return INFINITY;
        return sqrt(g.gamma * P / rho);
    };
    switch (var) {
    case HC_DISPLAY_RHO: return U[0];
    case HC_DISPLAY_MX: return U[1];
    case HC_DISPLAY_MY: return U[2];
    case HC_DISPLAY_MZ: return U[3];
    case HC_DISPLAY_M_MAG: return sqrt(lenSq3(U[1], U[2], U[3]));
    case HC_DISPLAY_ETOTAL: return U[4];
    case HC_DISPLAY_EPOT: return U[5];
    case HC_DISPLAY_VX: return vx;
    case HC_DISPLAY_VY: return vy;
    case HC_DISPLAY_VZ: return vz;
    case HC_DISPLAY_V_MAG: return sqrt(lenSq3(vx, vy, vz));
    case HC_DISPLAY_P: return P;
    case HC_DISPLAY_EINT_SPECIFIC: return (P / (g.gamma - 1.)) / rho;
    case HC_DISPLAY_EKIN_SPECIFIC: return .5 * lenSq3(vx, vy, vz);
    case HC_DISPLAY_ETOTAL_SPECIFIC: return U[4] / rho;
    case HC_DISPLAY_EINT: return P / (g.gamma - 1.);
    case HC_DISPLAY_EKIN: return rho * (.5 * lenSq3(vx, vy, vz));
    case HC_DISPLAY_EPOT_VOLUME: return U[0] * U[5];
    case HC_DISPLAY_S: return P / pow(rho, g.gamma);
    case HC_DISPLAY_H: return P * (g.gamma / (g.gamma - 1.));
    case HC_DISPLAY_H_SPECIFIC: return P * (g.gamma / (g.gamma - 1.)) / rho;
    case HC_DISPLAY_HTOTAL: return P + U[4];
    case HC_DISPLAY_HTOTAL_SPECIFIC: return (P + U[4]) / rho;
    case HC_DISPLAY_CS: return Cs();
    case HC_DISPLAY_MACH: return sqrt(lenSq3(vx, vy, vz)) / Cs();
    case HC_DISPLAY_TEMPERATURE:
        // calc_T = calc_eInt_fromCons / C_v (euler.cl:114-131)
        return ((U[4] - .5 * lenSq3(U[1], U[2], U[3]) / U[0]) / U[0] - U[5]) / kAirCv;
    default: return 0.;
    }
}

__device__ __forceinline__ const double* cellAt(const Grid& g, int i, int j, int k) {
    return g.U + 6 * (i * g.stride[0] + j * g.stride[1] + k * g.stride[2]);
}

__device__ __forceinline__ int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

// The display value of every cell of the grid (numGhost = 2 ghost layers on
// each active axis), x fastest.  T = double (the buffer) or float (the
// texture the image kernels sample).
template <typename T>
__global__ void k_display(Grid g, int var, int zeroBorder, T* out) {
    int const G = 2;
    int const fx = g.n[0] + (g.dim > 0 ? 2 * G : 0);
    int const fy = g.dim > 1 ? g.n[1] + 2 * G : 1;
    int const fz = g.dim > 2 ? g.n[2] + 2 * G : 1;
    long long const total = (long long)fx * fy * fz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
         c += (long long)gridDim.x * blockDim.x) {
        int const ix = (int)(c % fx), iy = (int)((c / fx) % fy), iz = (int)(c / ((long long)fx * fy));
        int f[3] = {ix, iy, iz};
        bool oob = false;
        int in[3] = {0, 0, 0};
        for (int d = 0; d < g.dim; ++d) {
            int const x = f[d] - G;
            oob = oob || x < 0 || x >= g.n[d];
            in[d] = clampi(x, 0, g.n[d] - 1);
        }
        double v = 0.;
        if (!(zeroBorder && oob)) v = displayValue(g, cellAt(g, in[0], in[1], in[2]), var);
        out[c] = (T)v;
    }
}

// Per-block partial min, max, sum over the interior, then sum of (x - mean)^2.
__global__ void k_range_partial(Grid g, int var, int pass, double mean, double* part) {
    __shared__ double smin[256], smax[256], ssum[256];
    long long const total = (long long)g.n[0] * g.n[1] * g.n[2];
    double mn = INFINITY, mx = -INFINITY, sm = 0.;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
         c += (long long)gridDim.x * blockDim.x) {
        int const i = (int)(c % g.n[0]), j = (int)((c / g.n[0]) % g.n[1]), k = (int)(c / ((long long)g.n[0] * g.n[1]));
        double const v = displayValue(g, cellAt(g, i, j, k), var);
        if (pass == 0) {
            mn = v < mn ? v : mn;
            mx = v > mx ? v : mx;
            sm += v;
        } else {
            double const d = v - mean;
            sm += d * d;
        }
    }
    smin[threadIdx.x] = mn;
    smax[threadIdx.x] = mx;
    ssum[threadIdx.x] = sm;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            double const a = smin[threadIdx.x + s], b = smax[threadIdx.x + s];
            smin[threadIdx.x] = a < smin[threadIdx.x] ? a : smin[threadIdx.x];
            smax[threadIdx.x] = b > smax[threadIdx.x] ? b : smax[threadIdx.x];
            ssum[threadIdx.x] += ssum[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x + 0] = smin[0];
        part[3 * blockIdx.x + 1] = smax[0];
        part[3 * blockIdx.x + 2] = ssum[0];
    }
}

// ---- palette and textures ---------------------------------------------------------

constexpr int kGradW = 1024;   // GLGradientTex2D(1024, colors, false), hydro/app.lua:1231

struct Palette {
    int n;
    float c[8][4];
};

// The palettes of hydro/draw/palette.lua that are written out there (the
// commented-out ones and the random palette are not).
static Palette palette_of(int which) {
    Palette p;
    std::memset(&p, 0, sizeof(p));
    auto set = [&](std::initializer_list<std::initializer_list<float>> cs) {
        p.n = 0;
        for (auto& c : cs) {
            int k = 0;
            for (float x : c) p.c[p.n][k++] = x;
            p.n++;
        }
    };
    switch (which) {
    case HC_PALETTE_STRIPES:
        // 32 entries alternating white, black (range(32):mapi(i -> ({black,
        // white})[i % 2 + 1]) starts at i = 1): the two stored, n < 0 marks
        // the 32-entry alternation for gradient_fill
        set({{1, 1, 1, 1}, {0, 0, 0, 0}});
        p.n = -32;
        break;
    case HC_PALETTE_BLUE: set({{0, 0, 0, .8f}, {.5f, .5f, 1, .8f}, {1, 1, 1, .8f}}); break;
    case HC_PALETTE_PARAVIEW:
        set({{0x3c / 255.f, 0x4e / 255.f, 0xc2 / 255.f, 1}, {0xdd / 255.f, 0xdd / 255.f, 0xdd / 255.f, 1},
             {0xb4 / 255.f, 0x04 / 255.f, 0x26 / 255.f, 1}});
        break;
    default:   // HC_PALETTE_WHITE_RAINBOW_BLACK
        set({{0, 0, 1, .8f}, {0, 1, 1, .8f}, {0, 1, 0, .8f}, {1, 1, 0, .8f}, {1, .5f, 0, .8f}, {1, 0, 0, .8f},
             {1, 1, 1, .8f}});
    }
    return p;
}

// The gradient texture: texel i at f = i / (W - 1) along the colour list,
// linear between neighbouring colours (the colours are not wrapped).  The
// texture class lives outside the reference (lua-gl's GLGradientTex2D); this
// is its documented behaviour, restated.
static void gradient_fill(const Palette& p, float* rgba) {
    int const n = p.n < 0 ? -p.n : p.n;
    for (int i = 0; i < kGradW; ++i) {
        double const f = (double)i / (kGradW - 1) * (n - 1);
        int lo = (int)std::floor(f);
        if (lo > n - 2) lo = n - 2;
        if (lo < 0) lo = 0;
        double const t = f - lo;
        for (int k = 0; k < 4; ++k) {
            int const a = p.n < 0 ? lo % 2 : lo, b = p.n < 0 ? (lo + 1) % 2 : lo + 1;
            rgba[4 * i + k] = (float)((1. - t) * p.c[a][k] + t * p.c[b][k]);
        }
    }
}

struct Tex {
    const float* v;       // texels, x fastest; `comps` floats each
    int w, h, d, comps;
};

__device__ __forceinline__ int wrapi(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}

// GL_LINEAR with GL_REPEAT at normalised coordinates (u, v, w); unused axes
// have size 1.
__device__ float4 sampleLinear(const Tex& t, float u, float v, float w) {
    float const x = u * t.w - .5f, y = v * t.h - .5f, z = w * t.d - .5f;
    float const fx = floorf(x), fy = floorf(y), fz = floorf(z);
    float const ax = x - fx, ay = y - fy, az = z - fz;
    int const x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
    float acc[4] = {0, 0, 0, 0};
    for (int dz = 0; dz < (t.d > 1 ? 2 : 1); ++dz)
        for (int dy = 0; dy < (t.h > 1 ? 2 : 1); ++dy)
            for (int dx = 0; dx < 2; ++dx) {
                float const wgt = (dx ? ax : 1.f - ax) * (t.h > 1 ? (dy ? ay : 1.f - ay) : 1.f) *
                                  (t.d > 1 ? (dz ? az : 1.f - az) : 1.f);
                long long const idx = wrapi(x0 + dx, t.w) +
                                      (long long)t.w * (wrapi(y0 + dy, t.h) + (long long)t.h * wrapi(z0 + dz, t.d));
                for (int k = 0; k < t.comps; ++k) acc[k] += wgt * t.v[idx * t.comps + k];
            }
    return make_float4(acc[0], acc[1], acc[2], acc[3]);
}

struct View {
    // draw.glsl uniforms
    int dim;                                  // displayDim
    float mins[3], maxs[3];                   // solverMins / solverMaxs
    float gridSize[3], sizeWithoutBorder[3];  // texture size with / without the ghosts
    float valueMin, valueMax;
    int useLog;
    float q[4];                               // displaySliceAngle (x, y, z, w)
    float fixedZ;                             // displayFixed.y
    float bbox[4];
    int width, height;
    // volume
    float eye[3], right[3], up[3], fwd[3], tanHalfFov;
    float alpha, alphaGamma, numIsobars;
    int maxIter, useIsobars, useLighting;
    // LIC
    int licIter, noiseSize;
    // slice stack
    int sliceAxis, numSlices;
};

__device__ __forceinline__ float3 quatRotate(const float* q, float3 v) {
    // draw.glsl:150-157: v + 2 q.xyz x (q.xyz x v + q.w v)
    float3 const u = make_float3(q[0], q[1], q[2]);
    float3 const t = make_float3(u.y * v.z - u.z * v.y + q[3] * v.x, u.z * v.x - u.x * v.z + q[3] * v.y,
                                 u.x * v.y - u.y * v.x + q[3] * v.z);
    return make_float3(v.x + 2.f * (u.y * t.z - u.z * t.y), v.y + 2.f * (u.z * t.x - u.x * t.z),
                       v.z + 2.f * (u.x * t.y - u.y * t.x));
}

// chartToTexCoord (draw.glsl:128-131): ghost-inclusive texture coordinates
__device__ __forceinline__ float3 chartToTex(const View& V, float3 x) {
    return make_float3(((x.x - V.mins[0]) / (V.maxs[0] - V.mins[0]) * V.sizeWithoutBorder[0] + 2.f) / V.gridSize[0],
                       ((x.y - V.mins[1]) / (V.maxs[1] - V.mins[1]) * V.sizeWithoutBorder[1] + 2.f) / V.gridSize[1],
                       ((x.z - V.mins[2]) / (V.maxs[2] - V.mins[2]) * V.sizeWithoutBorder[2] + 2.f) / V.gridSize[2]);
}

// texToNoGhostCoord (draw.glsl:133-135)
__device__ __forceinline__ float3 texToNoGhost(const View& V, float3 x) {
    return make_float3((x.x * V.sizeWithoutBorder[0] + 2.f) / V.gridSize[0],
                       (x.y * V.sizeWithoutBorder[1] + 2.f) / V.gridSize[1],
                       (x.z * V.sizeWithoutBorder[2] + 2.f) / V.gridSize[2]);
}

__device__ __forceinline__ float logmap(float x) { return logf(fabsf(x)) * (float)(1. / 2.302585092994046); }

// getGradientFrac (draw.glsl:52-71)
__device__ float gradientFrac(const View& V, float value) {
    if (V.useLog) {
        float lo = logmap(V.valueMin), hi = logmap(V.valueMax);
        if ((V.valueMin < 0.f) != (V.valueMax < 0.f)) {
            lo = 0.f;
        } else if (V.valueMin < 0.f) {
            float const t = lo;
            lo = hi;
            hi = t;
        }
        return (logmap(value) - lo) / (hi - lo);
    }
    return (value - V.valueMin) / (V.valueMax - V.valueMin);
}

// getGradientTexCoord + texture(gradientTex, ...) (draw.glsl:77-85)
__device__ float4 gradientColor(const Tex& grad, float frac) {
    float const tc = (frac * (float)(kGradW - 1) + .5f) * (1.f / kGradW);
    return sampleLinear(grad, tc, .5f, .5f);
}

__device__ __forceinline__ uchar4 toRGBA8(float4 c) {
    auto q = [](float x) -> unsigned char {
        x = x != x ? 0.f : fminf(fmaxf(x, 0.f), 1.f);
        return (unsigned char)__float2int_rn(x * 255.f);
    };
    return make_uchar4(q(c.x), q(c.y), q(c.z), q(c.w));
}

// the fragment of pixel (px, py) (row 0 at the bottom, as glReadPixels
// returns it) in the view rectangle bbox
__device__ __forceinline__ float3 viewCoordOf(const View& V, int px, int py) {
    float const sx = (px + .5f) / V.width, sy = (py + .5f) / V.height;
    return make_float3(V.bbox[0] + (V.bbox[2] - V.bbox[0]) * sx, V.bbox[1] + (V.bbox[3] - V.bbox[1]) * sy, 0.f);
}

__device__ __forceinline__ bool outside(const View& V, float3 t) {
    if (t.x < 0.f || t.x > 1.f) return true;
    if (V.dim > 1 && (t.y < 0.f || t.y > 1.f)) return true;
    if (V.dim > 2 && (t.z < 0.f || t.z > 1.f)) return true;
    return false;
}

// 2d_heatmap.glsl:28-59 (with the chart map the identity: Cartesian, display_useCoordMap)
__global__ void k_heatmap(View V, Tex tex, Tex grad, uchar4* out) {
    int const px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= V.width || py >= V.height) return;
    float3 chart = viewCoordOf(V, px, py);
    chart.z = V.fixedZ;
    chart = quatRotate(V.q, chart);
    float3 const tc = chartToTex(V, chart);
    uchar4 o = make_uchar4(0, 0, 0, 0);
    if (!outside(V, tc)) {
        float const value = sampleLinear(tex, tc.x, tc.y, tc.z).x;
        o = toRGBA8(gradientColor(grad, gradientFrac(V, value)));
    }
    out[(long long)py * V.width + px] = o;
}

__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
    float const t = fminf(fmaxf((x - e0) / (e1 - e0), 0.f), 1.f);
    return t * t * (3.f - 2.f * t);
}

// volumetric.glsl:36-110 with a pinhole camera in place of the cube's
// rasterisation: each pixel's ray enters the domain box at the point the
// cube face would have been drawn; from there the shader's march runs
// unchanged (its step is the normalised world direction over maxiter, taken
// in texture coordinates).  Lighting uses the world frame (normalMatrix = I).
__global__ void k_volume(View V, Tex tex, Tex grad, uchar4* out) {
    int const px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= V.width || py >= V.height) return;
    float const sx = ((px + .5f) / V.width * 2.f - 1.f) * V.tanHalfFov * ((float)V.width / V.height);
    float const sy = ((py + .5f) / V.height * 2.f - 1.f) * V.tanHalfFov;
    float3 dir = make_float3(V.fwd[0] + sx * V.right[0] + sy * V.up[0], V.fwd[1] + sx * V.right[1] + sy * V.up[1],
                             V.fwd[2] + sx * V.right[2] + sy * V.up[2]);
    // slab intersection with [mins, maxs]
    float t0 = 0.f, t1 = INFINITY;
    float const e[3] = {V.eye[0], V.eye[1], V.eye[2]};
    float const dv[3] = {dir.x, dir.y, dir.z};
    for (int a = 0; a < 3; ++a) {
        if (dv[a] == 0.f) {
            if (e[a] < V.mins[a] || e[a] > V.maxs[a]) t0 = INFINITY;
            continue;
        }
        float ta = (V.mins[a] - e[a]) / dv[a], tb = (V.maxs[a] - e[a]) / dv[a];
        if (ta > tb) { float const s = ta; ta = tb; tb = s; }
        t0 = fmaxf(t0, ta);
        t1 = fminf(t1, tb);
    }
    uchar4 o = make_uchar4(0, 0, 0, 0);
    if (t0 <= t1 && t0 < INFINITY) {
        float3 const start = make_float3(e[0] + t0 * dv[0], e[1] + t0 * dv[1], e[2] + t0 * dv[2]);
        float3 p = make_float3((start.x - V.mins[0]) / (V.maxs[0] - V.mins[0]),
                               (start.y - V.mins[1]) / (V.maxs[1] - V.mins[1]),
                               (start.z - V.mins[2]) / (V.maxs[2] - V.mins[2]));
        // getVoxelValue: [0,1] onto the interior texels
        auto voxel = [&](float3 q) -> float {
            float3 const tq = make_float3(q.x * (V.sizeWithoutBorder[0] / V.gridSize[0]) + 2.f / V.gridSize[0],
                                          q.y * (V.sizeWithoutBorder[1] / V.gridSize[1]) + 2.f / V.gridSize[1],
                                          q.z * (V.sizeWithoutBorder[2] / V.gridSize[2]) + 2.f / V.gridSize[2]);
            return sampleLinear(tex, tq.x, tq.y, tq.z).x;
        };
        float rgb[3] = {0.f, 0.f, 0.f}, ra = 1.f;
        float value = voxel(p);
        float frac = gradientFrac(V, value);
        float4 c = gradientColor(grad, frac);
        float a = V.alpha * fminf(1.f, sqrtf(c.x * c.x + c.y * c.y + c.z * c.z));
        rgb[0] += ra * a * c.x;
        rgb[1] += ra * a * c.y;
        rgb[2] += ra * a * c.z;
        ra *= 1.f - a;
        float3 const d = make_float3(start.x - V.eye[0], start.y - V.eye[1], start.z - V.eye[2]);
        float const inv = 1.f / (sqrtf(d.x * d.x + d.y * d.y + d.z * d.z) * (float)V.maxIter);
        float3 const step = make_float3(d.x * inv, d.y * inv, d.z * inv);
        for (int i = 2; i <= V.maxIter; ++i) {
            p = make_float3(p.x + step.x, p.y + step.y, p.z + step.z);
            if (p.x < 0.f || p.y < 0.f || p.z < 0.f || p.x > 1.f || p.y > 1.f || p.z > 1.f) break;
            value = voxel(p);
            frac = gradientFrac(V, value);
            c = gradientColor(grad, frac);
            if (V.useIsobars) {
                float const ff = frac * V.numIsobars + .5f;
                float const ffrac = ff - floorf(ff);
                float const th = .1f;
                a = smoothstepf(0.f, th / 3.f, ffrac) - smoothstepf(2.f / 3.f * th, th, ffrac);
            } else {
                a = powf(V.alpha, V.alphaGamma);
            }
            if (V.useLighting) {
                float const h = 1.f / 32.f, ambient = .3f;
                float gx = voxel(make_float3(p.x + h, p.y, p.z)) - voxel(make_float3(p.x - h, p.y, p.z));
                float gy = voxel(make_float3(p.x, p.y + h, p.z)) - voxel(make_float3(p.x, p.y - h, p.z));
                float gz = voxel(make_float3(p.x, p.y, p.z + h)) - voxel(make_float3(p.x, p.y, p.z - h));
                float const gl = sqrtf(gx * gx + gy * gy + gz * gz);
                float const ld = fabsf(gz / gl);   // light along +z
                // GLSL max(x, y) = x < y ? y : x: a flat region (0/0) gives the ambient term
                float const lum = ambient < ld ? ld : ambient;
                c.x *= lum;
                c.y *= lum;
                c.z *= lum;
            }
            rgb[0] += ra * a * c.x;
            rgb[1] += ra * a * c.y;
            rgb[2] += ra * a * c.z;
            ra *= 1.f - a;
        }
        o = toRGBA8(make_float4(rgb[0], rgb[1], rgb[2], 1.f - ra));
    }
    out[(long long)py * V.width + px] = o;
}

// The volume as 3d_slice.lua draws it: num_slices + 1 quads across the grid
// along the view axis (the one the camera looks most along), blended back to
// front with (SRC_ALPHA, ONE_MINUS_SRC_ALPHA) onto a clear (0, 0, 0, 0)
// framebuffer; here an orthographic view along the axis, the image spanning
// the other two (in x, y, z order).  Each slice's fragment is 3d_slice.glsl's
// (voxel through the palette; alpha pow(alpha, alphaGamma) or the isobar
// profile; optional lighting) with the projection factor 1 / (-n.w) taken as
// 1 (it belongs to the GL camera, which has no headless counterpart), then
// times alpha.
__global__ void k_slices(View V, Tex tex, Tex grad, uchar4* out) {
    int const px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= V.width || py >= V.height) return;
    int const axis = V.sliceAxis % 3;
    bool const towardsPlus = V.sliceAxis < 3;
    int const a1 = axis == 0 ? 1 : 0, a2 = axis == 2 ? 1 : 2;
    float const u = (px + .5f) / V.width, v = (py + .5f) / V.height;
    int const n = V.numSlices;
    float rgb[3] = {0.f, 0.f, 0.f}, acc = 0.f;
    for (int s = 0; s <= n; ++s) {
        // back to front: looking towards +axis the back is f = 1
        int const j = towardsPlus ? n - s : s;
        float const f = (float)j / (float)n;
        float c3[3];
        c3[axis] = f;
        c3[a1] = u;
        c3[a2] = v;
        // with the chart map the identity the world coordinate of a slice
        // point maps back to these texture coordinates; the slice rotation
        // is applied about them as the shader does
        float3 tc = quatRotate(V.q, make_float3(c3[0], c3[1], c3[2]));
        if (tc.x < 0.f || tc.x > 1.f || tc.y < 0.f || tc.y > 1.f || tc.z < 0.f || tc.z > 1.f) continue;
        float3 const ng = texToNoGhost(V, tc);
        auto voxel = [&](float3 q) { return sampleLinear(tex, q.x, q.y, q.z).x; };
        float const value = voxel(ng);
        float const frac = gradientFrac(V, value);
        float4 c = gradientColor(grad, frac);
        float a;
        if (V.useIsobars) {
            float const ff = frac * V.numIsobars + .5f;
            float const ffrac = ff - floorf(ff);
            float const th = .1f;
            a = smoothstepf(0.f, th / 3.f, ffrac) - smoothstepf(2.f / 3.f * th, th, ffrac);
        } else {
            a = powf(V.alpha, V.alphaGamma);
        }
        if (V.useLighting) {
            float const h = 1.f / 32.f, ambient = .3f;
            float gx = voxel(make_float3(ng.x + h, ng.y, ng.z)) - voxel(make_float3(ng.x - h, ng.y, ng.z));
            float gy = voxel(make_float3(ng.x, ng.y + h, ng.z)) - voxel(make_float3(ng.x, ng.y - h, ng.z));
            float gz = voxel(make_float3(ng.x, ng.y, ng.z + h)) - voxel(make_float3(ng.x, ng.y, ng.z - h));
            float const ld = fabsf(gz / sqrtf(gx * gx + gy * gy + gz * gz));
            float const lum = ambient < ld ? ld : ambient;   // GLSL max(x, y) = x < y ? y : x
            c.x *= lum;
            c.y *= lum;
            c.z *= lum;
        }
        float const sa = a * V.alpha;
        rgb[0] = c.x * sa + rgb[0] * (1.f - sa);
        rgb[1] = c.y * sa + rgb[1] * (1.f - sa);
        rgb[2] = c.z * sa + rgb[2] * (1.f - sa);
        acc = sa * sa + acc * (1.f - sa);
    }
    out[(long long)py * V.width + px] = toRGBA8(make_float4(rgb[0], rgb[1], rgb[2], acc));
}

// vector_lic.glsl:36-107 over the velocity (the 'v' display variable), the
// noise texture a seeded uniform field (vector_lic.lua:69-88 fills it with
// math.random).  ds = 1 / noiseSize; chartToNoGhostCoord applies the ghost
// offset on top of chartToTexCoord, as draw.glsl:137-139 does.
__global__ void k_lic(View V, Tex vel, Tex noise, Tex grad, uchar4* out) {
    int const px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= V.width || py >= V.height) return;
    float3 chart = viewCoordOf(V, px, py);
    chart.z = V.fixedZ;
    chart = quatRotate(V.q, chart);
    float3 const tc = chartToTex(V, chart);
    uchar4 o = make_uchar4(0, 0, 0, 0);
    if (!outside(V, tc)) {
        auto noGhost = [&](float3 x) { return texToNoGhost(V, chartToTex(V, x)); };
        float3 const ng = noGhost(chart);
        float lic = sampleLinear(noise, ng.x, ng.y, .5f).x;
        float total = 1.f;
        float const ds = 1.f / V.noiseSize;
        for (int dir = -1; dir <= 1; dir += 2) {
            float3 pos = chart;
            float3 last = make_float3(0.f, 0.f, 0.f);
            for (int it = 0; it < V.licIter; ++it) {
                float3 const q = noGhost(pos);
                float4 const u = sampleLinear(vel, q.x, q.y, q.z);
                if (it > 0 && u.x * last.x + u.y * last.y + u.z * last.z < 0.f) break;
                float const m = sqrtf(u.x * u.x + u.y * u.y + u.z * u.z);
                if (m == 0.f) break;
                float const s = ds * dir / m;
                pos = make_float3(pos.x + u.x * s, pos.y + u.y * s, pos.z + u.z * s);
                float const f = (float)(it + 1) / (float)(V.licIter + 1);
                float const w = smoothstepf(1.f, 0.f, f);
                float3 const qn = noGhost(pos);
                lic += sampleLinear(noise, qn.x, qn.y, .5f).x * w;
                total += w;
                last = make_float3(u.x, u.y, u.z);
            }
        }
        lic /= total;
        lic = smoothstepf(.2f, .8f, lic);
        float4 const u0 = sampleLinear(vel, ng.x, ng.y, ng.z);
        float mag = sqrtf(u0.x * u0.x + u0.y * u0.y + u0.z * u0.z);
        mag = fminf(fmaxf(mag, V.valueMin), V.valueMax);
        float4 c = gradientColor(grad, gradientFrac(V, mag));
        c.x *= lic;
        c.y *= lic;
        c.z *= lic;
        o = toRGBA8(c);
    }
    out[(long long)py * V.width + px] = o;
}

// velocity texels (v.x, v.y, v.z) over the ghost-inclusive grid (ghosts show
// the nearest interior cell)
__global__ void k_velocity(Grid g, float* out) {
    int const G = 2;
    int const fx = g.n[0] + 2 * G;
    int const fy = g.dim > 1 ? g.n[1] + 2 * G : 1;
    int const fz = g.dim > 2 ? g.n[2] + 2 * G : 1;
    long long const total = (long long)fx * fy * fz;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < total;
         c += (long long)gridDim.x * blockDim.x) {
        int f[3] = {(int)(c % fx), (int)((c / fx) % fy), (int)(c / ((long long)fx * fy))};
        int in[3] = {0, 0, 0};
        for (int d = 0; d < g.dim; ++d) in[d] = clampi(f[d] - G, 0, g.n[d] - 1);
        const double* U = cellAt(g, in[0], in[1], in[2]);
        double const inv = 1. / U[0];
        out[4 * c + 0] = (float)(U[1] * inv);
        out[4 * c + 1] = (float)(U[2] * inv);
        out[4 * c + 2] = (float)(U[3] * inv);
        out[4 * c + 3] = 0.f;
    }
}

// noise texels: the k-th uniform of SplitMix64(seed)
__global__ void k_noise(unsigned long long seed, long long n, float* out) {
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
        unsigned long long z = seed + ((unsigned long long)k + 1ull) * 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z = z ^ (z >> 31);
        out[k] = (float)((double)(z >> 11) * (1.0 / 9007199254740992.0));
    }
}

unsigned blocks_for(long long n) {
    long long b = (n + 255) / 256;
    return (unsigned)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

}  // namespace viz

// ---- host side --------------------------------------------------------------------

namespace {

viz::Grid grid_of(const VizState& st) {
    viz::Grid g;
    g.U = st.U;
    for (int k = 0; k < 3; ++k) {
        g.stride[k] = st.stride[k];
        g.n[k] = k < st.d.dim ? st.d.n[k] : 1;
        g.mins[k] = st.d.mins[k];
        g.maxs[k] = st.d.maxs[k];
    }
    g.dim = st.d.dim;
    g.gamma = st.d.gamma;
    g.rhoMin = st.d.rho_min;
    g.PMin = st.d.p_min;
    return g;
}

long long full_cells_of(const hc_solver_desc& d) {
    long long n = 1;
    for (int k = 0; k < d.dim; ++k) n *= d.n[k] + 4;
    return n;
}

}  // namespace

int viz_display(const VizState& st, int var, int zero_border, double* out_dev, cudaStream_t s) {
    if (var < 0 || var >= HC_NUM_DISPLAY_VARS) return fail(HC_ERR_INVALID, "unknown display variable");
    viz::Grid const g = grid_of(st);
    viz::k_display<double><<<viz::blocks_for(full_cells_of(st.d)), 256, 0, s>>>(g, var, zero_border, out_dev);
    HC_CUDA(cudaGetLastError());
    return HC_OK;
}

int viz_range(const VizState& st, int var, double out[4], cudaStream_t s) {
    if (var < 0 || var >= HC_NUM_DISPLAY_VARS) return fail(HC_ERR_INVALID, "unknown display variable");
    viz::Grid const g = grid_of(st);
    long long const n = (long long)g.n[0] * g.n[1] * g.n[2];
    int const blocks = (int)viz::blocks_for(n) > 1024 ? 1024 : (int)viz::blocks_for(n);
    double* part = nullptr;
    HC_CUDA(cudaMalloc(&part, (size_t)blocks * 3 * sizeof(double)));
    std::vector<double> h((size_t)blocks * 3);
    int r = HC_OK;
    double mn = INFINITY, mx = -INFINITY, sum = 0., dev = 0.;
    for (int pass = 0; pass < 2 && r == HC_OK; ++pass) {
        double const mean = sum / (double)n;
        viz::k_range_partial<<<blocks, 256, 0, s>>>(g, var, pass, mean, part);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) { r = cuda_fail(e, "display range"); break; }
        double acc = 0.;
        for (int b = 0; b < blocks; ++b) {
            if (pass == 0) {
                mn = h[3 * b] < mn ? h[3 * b] : mn;
                mx = h[3 * b + 1] > mx ? h[3 * b + 1] : mx;
            }
            acc += h[3 * b + 2];
        }
        if (pass == 0) sum = acc;
        else dev = acc;
    }
    cudaFree(part);
    if (r != HC_OK) return r;
    out[0] = mn;
    out[1] = mx;
    out[2] = sum / (double)n;
    out[3] = std::sqrt(dev / (double)n);
    return HC_OK;
}

int viz_render(const VizState& st, const hc_render& R, unsigned char* out_dev, cudaStream_t s) {
    if (R.width <= 0 || R.height <= 0 || (long long)R.width * R.height > (1ll << 28))
        return fail(HC_ERR_INVALID, "image size");
    if (R.mode < HC_RENDER_HEATMAP || R.mode > HC_RENDER_SLICES) return fail(HC_ERR_INVALID, "render mode");
    if (R.var < 0 || R.var >= HC_NUM_DISPLAY_VARS) return fail(HC_ERR_INVALID, "unknown display variable");
    if ((R.mode == HC_RENDER_VOLUME || R.mode == HC_RENDER_SLICES) && st.d.dim != 3)
        return fail(HC_ERR_INVALID, "the volume and slice views need a 3D grid");
    if (R.mode == HC_RENDER_SLICES && (R.num_slices < 1 || R.num_slices > 4096 || R.slice_axis < 0 || R.slice_axis > 5))
        return fail(HC_ERR_INVALID, "num_slices / slice_axis");
    if (R.mode == HC_RENDER_LIC && st.d.dim < 2) return fail(HC_ERR_INVALID, "the LIC view needs a 2D or 3D grid");
    if (R.mode != HC_RENDER_HEATMAP && R.max_iter > 4096) return fail(HC_ERR_INVALID, "max_iter");
    viz::Grid const g = grid_of(st);
    double range[4] = {R.value_min, R.value_max, 0, 0};
    if (!(R.value_min < R.value_max)) {
        int const var = R.mode == HC_RENDER_LIC ? HC_DISPLAY_V_MAG : R.var;
        HC_CHECK(viz_range(st, var, range, s));
    }
    viz::View V;
    std::memset(&V, 0, sizeof(V));
    V.dim = st.d.dim;
    for (int k = 0; k < 3; ++k) {
        bool const act = k < st.d.dim;
        V.mins[k] = (float)st.d.mins[k];
        V.maxs[k] = (float)st.d.maxs[k];
        V.gridSize[k] = act ? (float)(st.d.n[k] + 4) : 1.f;
        V.sizeWithoutBorder[k] = act ? (float)st.d.n[k] : 1.f;
    }
    // the texture of an unused axis has size 1 and numGhost 0 along it
    for (int k = st.d.dim; k < 3; ++k) {
        V.gridSize[k] = 5.f;   // (x * 1 + 2) / 5 stays inside [0, 1] for any x in [0, 1]
        V.sizeWithoutBorder[k] = 1.f;
    }
    V.valueMin = (float)range[0];
    V.valueMax = (float)range[1];
    V.useLog = R.use_log;
    double qn = std::sqrt(R.slice_angle[0] * R.slice_angle[0] + R.slice_angle[1] * R.slice_angle[1] +
                          R.slice_angle[2] * R.slice_angle[2] + R.slice_angle[3] * R.slice_angle[3]);
    if (!(qn > 0)) return fail(HC_ERR_INVALID, "slice_angle is not a rotation");
    for (int k = 0; k < 4; ++k) V.q[k] = (float)(R.slice_angle[k] / qn);
    V.fixedZ = (float)R.fixed_z;
    for (int k = 0; k < 4; ++k) V.bbox[k] = (float)R.bbox[k];
    if (!(R.bbox[0] != R.bbox[2] && R.bbox[1] != R.bbox[3])) {
        V.bbox[0] = (float)st.d.mins[0];
        V.bbox[1] = st.d.dim > 1 ? (float)st.d.mins[1] : -1.f;
        V.bbox[2] = (float)st.d.maxs[0];
        V.bbox[3] = st.d.dim > 1 ? (float)st.d.maxs[1] : 1.f;
    }
    V.width = R.width;
    V.height = R.height;
    V.alpha = (float)R.alpha;
    V.alphaGamma = (float)R.alpha_gamma;
    V.numIsobars = (float)R.num_isobars;
    V.maxIter = R.max_iter;
    V.useIsobars = R.use_isobars;
    V.useLighting = R.use_lighting;
    V.licIter = R.lic_iter;
    V.noiseSize = R.noise_size;
    V.sliceAxis = R.slice_axis;
    V.numSlices = R.num_slices;
    if (R.mode == HC_RENDER_VOLUME) {
        // camera: at `eye`, looking at the domain's centre, y up
        double c[3], f[3], up[3] = {0, 1, 0}, rt[3], u[3];
        for (int k = 0; k < 3; ++k) {
            c[k] = .5 * (st.d.mins[k] + st.d.maxs[k]);
            f[k] = c[k] - R.eye[k];
            V.eye[k] = (float)R.eye[k];
        }
        double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
        if (!(fl > 0)) return fail(HC_ERR_INVALID, "eye at the domain's centre");
        for (int k = 0; k < 3; ++k) f[k] /= fl;
        if (std::fabs(f[1]) > .999) { up[1] = 0; up[2] = 1; }
        rt[0] = f[1] * up[2] - f[2] * up[1];
        rt[1] = f[2] * up[0] - f[0] * up[2];
        rt[2] = f[0] * up[1] - f[1] * up[0];
        double rl = std::sqrt(rt[0] * rt[0] + rt[1] * rt[1] + rt[2] * rt[2]);
        for (int k = 0; k < 3; ++k) rt[k] /= rl;
        u[0] = rt[1] * f[2] - rt[2] * f[1];
        u[1] = rt[2] * f[0] - rt[0] * f[2];
        u[2] = rt[0] * f[1] - rt[1] * f[0];
        for (int k = 0; k < 3; ++k) {
            V.fwd[k] = (float)f[k];
            V.right[k] = (float)rt[k];
            V.up[k] = (float)u[k];
        }
        V.tanHalfFov = (float)std::tan(R.fov_y * M_PI / 360.);
        if (!(R.max_iter >= 2)) return fail(HC_ERR_INVALID, "max_iter");
    }
    if (R.mode == HC_RENDER_LIC && (R.lic_iter < 0 || R.lic_iter > 1024 || R.noise_size < 2 || R.noise_size > 8192))
        return fail(HC_ERR_INVALID, "lic_iter / noise_size");

    long long const nfull = full_cells_of(st.d);
    int const tw = st.d.n[0] + 4, th = st.d.dim > 1 ? st.d.n[1] + 4 : 1, td = st.d.dim > 2 ? st.d.n[2] + 4 : 1;
    viz::Palette const pal = viz::palette_of(R.palette);
    std::vector<float> gradHost(4 * viz::kGradW);
    viz::gradient_fill(pal, gradHost.data());
    size_t const texFloats = R.mode == HC_RENDER_LIC ? (size_t)nfull * 4 : (size_t)nfull;
    size_t const noiseFloats = R.mode == HC_RENDER_LIC ? (size_t)R.noise_size * R.noise_size : 0;
    void* scratch = nullptr;
    HC_CUDA(cudaMalloc(&scratch, (texFloats + noiseFloats + 4 * viz::kGradW) * sizeof(float)));
    float* texBuf = static_cast<float*>(scratch);
    float* noiseBuf = texBuf + texFloats;
    float* gradBuf = noiseBuf + noiseFloats;
    int r = HC_OK;
    cudaError_t e = cudaMemcpyAsync(gradBuf, gradHost.data(), gradHost.size() * sizeof(float), cudaMemcpyHostToDevice, s);
    viz::Tex grad{gradBuf, viz::kGradW, 1, 1, 4};
    dim3 const blk(16, 16), grd((R.width + 15) / 16, (R.height + 15) / 16);
    if (e == cudaSuccess) {
        if (R.mode == HC_RENDER_LIC) {
            viz::k_velocity<<<viz::blocks_for(nfull), 256, 0, s>>>(g, texBuf);
            viz::k_noise<<<viz::blocks_for((long long)noiseFloats), 256, 0, s>>>(R.noise_seed, (long long)noiseFloats,
                                                                                  noiseBuf);
            viz::Tex vel{texBuf, tw, th, td, 4};
            viz::Tex noise{noiseBuf, R.noise_size, R.noise_size, 1, 1};
            viz::k_lic<<<grd, blk, 0, s>>>(V, vel, noise, grad, reinterpret_cast<uchar4*>(out_dev));
        } else {
            viz::k_display<float><<<viz::blocks_for(nfull), 256, 0, s>>>(g, R.var, 0, texBuf);
            viz::Tex tex{texBuf, tw, th, td, 1};
            if (R.mode == HC_RENDER_HEATMAP) viz::k_heatmap<<<grd, blk, 0, s>>>(V, tex, grad, reinterpret_cast<uchar4*>(out_dev));
            else if (R.mode == HC_RENDER_SLICES) viz::k_slices<<<grd, blk, 0, s>>>(V, tex, grad, reinterpret_cast<uchar4*>(out_dev));
            else viz::k_volume<<<grd, blk, 0, s>>>(V, tex, grad, reinterpret_cast<uchar4*>(out_dev));
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) r = cuda_fail(e, "render");
    cudaFree(scratch);
    return r;
}

}  // namespace hc

extern "C" int hc_render_defaults(int mode, hc_render* out) {
    using namespace hc;
    if (!out) return fail(HC_ERR_INVALID, "out is NULL");
    if (mode < HC_RENDER_HEATMAP || mode > HC_RENDER_SLICES) return fail(HC_ERR_INVALID, "render mode");
    hc_render r;
    std::memset(&r, 0, sizeof(r));
    r.mode = mode;
    r.var = HC_DISPLAY_RHO;
    r.width = 512;
    r.height = 512;
    r.palette = HC_PALETTE_WHITE_RAINBOW_BLACK;
    r.slice_angle[3] = 1.;       // quatf(0,0,0,1), hydro/app.lua:813
    r.eye[0] = 2.;               // volume camera
    r.eye[1] = 1.5;
    r.eye[2] = 3.;
    r.fov_y = 45.;
    r.alpha = .15;               // volumetric / 3d_slice alpha and gamma
    r.alpha_gamma = 1.;
    r.max_iter = 100;
    r.num_isobars = 10.;
    r.lic_iter = 10;             // DrawVectorLIC.integralMaxIter, vector_lic.lua:12
    r.noise_size = 1024;         // HydroCLApp.drawVectorLICNoiseSize, app.lua:677
    r.noise_seed = 1;
    r.slice_axis = 2;            // looking along +z
    r.num_slices = 255;          // Draw3DSlice.numSlices, 3d_slice.lua
    if (mode == HC_RENDER_SLICES) {
        r.use_isobars = 1;       // Draw3DSlice.useIsos
        r.num_isobars = 20.;     // Draw3DSlice.numIsobars
    }
    *out = r;
    return HC_OK;
}
