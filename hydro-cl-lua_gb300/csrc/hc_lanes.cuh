// hc_lanes.cuh -- the fast (FP32) form of the Roe / PLM arithmetic written once
// for one lane (float) or two lanes (float2).
//
// Blackwell executes FP32 add / multiply / fused multiply-add on register
// pairs (__fadd2_rn, __fmul2_rn, __ffma2_rn: one instruction for two
// results).  A stage kernel that sweeps two neighbouring grid lines in
// lockstep evaluates both lines' interfaces with these packed operations;
// reciprocals, square roots, comparisons and selects stay per lane.
//
// Every operation here rounds once, exactly as written (explicitly rounded
// intrinsics; nothing is left for the compiler to contract into FMAs), so the
// one-lane and the two-lane instantiations, and every tile schedule of
// either, produce identical bits.  The mathematics is that of
// hc_fast_math.cuh (the reference's eigen-decomposition restated in the
// interface frame, the flux-split Roe flux without a flux limiter, the
// closed-form PLM half slopes); the rare branches (vacuum states) are
// evaluated lane by lane.
#pragma once

#include <cuda_runtime.h>

#include "hc_fast_math.cuh"

namespace hc {
namespace lanes {

// ---- per-lane masks -------------------------------------------------------

struct B2 { bool x, y; };

__device__ __forceinline__ bool any(bool m) { return m; }
__device__ __forceinline__ bool any(B2 m) { return m.x || m.y; }
__device__ __forceinline__ B2 operator||(B2 a, B2 b) { return {a.x || b.x, a.y || b.y}; }

template <typename V> struct MaskOf;
template <> struct MaskOf<float> { using type = bool; };
template <> struct MaskOf<float2> { using type = B2; };
template <typename V> using Mask = typename MaskOf<V>::type;

// ---- arithmetic (one rounding per operation) -------------------------------

template <typename V> __device__ __forceinline__ V splat(float x);
template <> __device__ __forceinline__ float splat<float>(float x) { return x; }
template <> __device__ __forceinline__ float2 splat<float2>(float x) { return make_float2(x, x); }

__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// c - a b
__device__ __forceinline__ float fnms(float a, float b, float c) { return __fmaf_rn(-a, b, c); }

__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b = a + (-1) b, rounded once
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 fnms(float2 a, float2 b, float2 c) { return __ffma2_rn(make_float2(-a.x, -a.y), b, c); }

// ---- per-lane operations ----------------------------------------------------

__device__ __forceinline__ float rcp(float x) { return __fdividef(1.f, x); }
__device__ __forceinline__ float rsq(float x) { return rsqrtf(x); }
__device__ __forceinline__ float sqr(float x) { return sqrtf(x); }
__device__ __forceinline__ float absv(float x) { return fabsf(x); }
__device__ __forceinline__ float vmax(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float vmin(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float sel(bool m, float a, float b) { return m ? a : b; }
__device__ __forceinline__ bool lt(float a, float b) { return a < b; }
__device__ __forceinline__ bool gt(float a, float b) { return a > b; }
__device__ __forceinline__ bool le(float a, float b) { return a <= b; }

__device__ __forceinline__ float2 rcp(float2 x) { return make_float2(rcp(x.x), rcp(x.y)); }
__device__ __forceinline__ float2 rsq(float2 x) { return make_float2(rsq(x.x), rsq(x.y)); }
__device__ __forceinline__ float2 sqr(float2 x) { return make_float2(sqr(x.x), sqr(x.y)); }
__device__ __forceinline__ float2 absv(float2 x) { return make_float2(fabsf(x.x), fabsf(x.y)); }
__device__ __forceinline__ float2 vmax(float2 x, float2 y) { return make_float2(vmax(x.x, y.x), vmax(x.y, y.y)); }
__device__ __forceinline__ float2 vmin(float2 x, float2 y) { return make_float2(vmin(x.x, y.x), vmin(x.y, y.y)); }
__device__ __forceinline__ float2 sel(B2 m, float2 a, float2 b) { return make_float2(m.x ? a.x : b.x, m.y ? a.y : b.y); }
__device__ __forceinline__ B2 lt(float2 a, float2 b) { return {a.x < b.x, a.y < b.y}; }
__device__ __forceinline__ B2 gt(float2 a, float2 b) { return {a.x > b.x, a.y > b.y}; }
__device__ __forceinline__ B2 le(float2 a, float2 b) { return {a.x <= b.x, a.y <= b.y}; }

__device__ __forceinline__ float lane(float v, int) { return v; }
__device__ __forceinline__ float lane(float2 v, int k) { return k ? v.y : v.x; }
__device__ __forceinline__ void setLane(float& v, int, float x) { v = x; }
__device__ __forceinline__ void setLane(float2& v, int k, float x) { if (k) v.y = x; else v.x = x; }
template <typename V> constexpr int nlanes() { return sizeof(V) / sizeof(float); }

// ---- states and eigen-structure ---------------------------------------------

struct Eos {
    float gamma, g1, rhoMin, PMin;
};

// A conserved state in the interface frame: rho, m_n, m_t1, m_t2, ETotal.
template <typename V> struct C5 { V u[5]; };

template <typename V> struct Eig {
    V vn, vt1, vt2, hT, Cs;
    V hvSq;          // |v|^2 / 2
    V invD, invD2;   // 1 / (2 Cs^2), 2 / (2 Cs^2)
    Mask<V> ident;   // rho < rhoMin: the transforms are the identity
};

// The Roe average with both sides above the vacuum threshold
// (euler.cl:347-430): one reciprocal square root per side gives
// sqrt(rho) = rho rs, 1/rho = rs^2 and the Roe weights.
template <typename V>
__device__ __forceinline__ V eigenRoe(Eig<V>& e, const Eos& s, const C5<V>& UL, const C5<V>& UR) {
    V const half = splat<V>(.5f), g1 = splat<V>(s.g1), rhoMin = splat<V>(s.rhoMin), zero = splat<V>(0.f);
    V const rsL = rsq(UL.u[0]), rsR = rsq(UR.u[0]);
    V const invL = mul(rsL, rsL), invR = mul(rsR, rsR);
    V const sL = mul(UL.u[0], rsL), sR = mul(UR.u[0], rsR);
    V const m2L = fma(UL.u[3], UL.u[3], fma(UL.u[2], UL.u[2], mul(UL.u[1], UL.u[1])));
    V const m2R = fma(UR.u[3], UR.u[3], fma(UR.u[2], UR.u[2], mul(UR.u[1], UR.u[1])));
    V const PL = sel(lt(UL.u[0], rhoMin), zero, mul(g1, fnms(mul(half, m2L), invL, UL.u[4])));
    V const PR = sel(lt(UR.u[0], rhoMin), zero, mul(g1, fnms(mul(half, m2R), invR, UR.u[4])));
    V const invDen = rcp(add(sL, sR));
    e.vn = mul(fma(UL.u[1], rsL, mul(UR.u[1], rsR)), invDen);
    e.vt1 = mul(fma(UL.u[2], rsL, mul(UR.u[2], rsR)), invDen);
    e.vt2 = mul(fma(UL.u[3], rsL, mul(UR.u[3], rsR)), invDen);
    V const hT = mul(fma(add(PL, UL.u[4]), rsL, mul(add(PR, UR.u[4]), rsR)), invDen);
    V const eKin = mul(half, fma(e.vt2, e.vt2, fma(e.vt1, e.vt1, mul(e.vn, e.vn))));
    e.hvSq = eKin;
    V const h = sub(hT, eKin);
    auto const low = lt(h, splat<V>(1e-5f));
    e.hT = sel(low, eKin, hT);
    e.Cs = sel(low, zero, sqr(mul(g1, h)));
    return mul(sL, sR);   // the averaged density
}

// One side at the vacuum threshold (or both): the other side's state, or zero.
__device__ __forceinline__ float eigenVac(Eig<float>& e, const Eos& s, const C5<float>& UL, const C5<float>& UR,
                                          bool lv, bool rv) {
    if (lv && rv) {
        e.vn = e.vt1 = e.vt2 = e.hvSq = e.hT = e.Cs = 0.f;
        return 0.f;
    }
    const C5<float>& Uo = lv ? UR : UL;
    float const inv = rcp(Uo.u[0]);
    float const m2 = fma(Uo.u[3], Uo.u[3], fma(Uo.u[2], Uo.u[2], mul(Uo.u[1], Uo.u[1])));
    bool const below = Uo.u[0] < s.rhoMin;
    float const P = below ? 0.f : mul(s.g1, fnms(mul(.5f, m2), inv, Uo.u[4]));
    e.vn = mul(Uo.u[1], inv);
    e.vt1 = mul(Uo.u[2], inv);
    e.vt2 = mul(Uo.u[3], inv);
    e.hvSq = mul(.5f, fma(e.vt2, e.vt2, fma(e.vt1, e.vt1, mul(e.vn, e.vn))));
    e.hT = mul(add(P, Uo.u[4]), inv);
    e.Cs = P <= s.PMin ? 0.f : (below ? __int_as_float(0x7f800000) : sqr(mul(mul(s.gamma, P), inv)));
    return Uo.u[0];
}

template <typename V>
__device__ __forceinline__ void finishEig(Eig<V>& e, const Eos& s, V rho) {
    e.ident = lt(rho, splat<V>(s.rhoMin));
    e.invD = rcp(mul(mul(splat<V>(2.f), e.Cs), e.Cs));
    e.invD2 = mul(splat<V>(2.f), e.invD);
}

__device__ __forceinline__ void eigen(Eig<float>& e, const Eos& s, const C5<float>& UL, const C5<float>& UR) {
    bool const lv = UL.u[0] < 1e-5f, rv = UR.u[0] < 1e-5f;
    float const rho = (lv || rv) ? eigenVac(e, s, UL, UR, lv, rv) : eigenRoe(e, s, UL, UR);
    finishEig(e, s, rho);
}

__device__ __forceinline__ void eigen(Eig<float2>& e, const Eos& s, const C5<float2>& UL, const C5<float2>& UR) {
    B2 const lv = lt(UL.u[0], splat<float2>(1e-5f)), rv = lt(UR.u[0], splat<float2>(1e-5f));
    if (!any(lv || rv)) {
        float2 const rho = eigenRoe(e, s, UL, UR);
        finishEig(e, s, rho);
        return;
    }
    // a vacuum side in either lane: each lane on its own
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        C5<float> l, r;
#pragma unroll
        for (int j = 0; j < 5; ++j) { l.u[j] = lane(UL.u[j], k); r.u[j] = lane(UR.u[j], k); }
        Eig<float> e1;
        eigen(e1, s, l, r);
        setLane(e.vn, k, e1.vn);
        setLane(e.vt1, k, e1.vt1);
        setLane(e.vt2, k, e1.vt2);
        setLane(e.hT, k, e1.hT);
        setLane(e.Cs, k, e1.Cs);
        setLane(e.hvSq, k, e1.hvSq);
        setLane(e.invD, k, e1.invD);
        setLane(e.invD2, k, e1.invD2);
        if (k) e.ident.y = e1.ident; else e.ident.x = e1.ident;
    }
}

// Lanes whose transforms are the identity take X unchanged.
template <typename V>
__device__ __forceinline__ void identLanes(V* out, const Eig<V>& e, const V* X) {
    if (any(e.ident)) {
#pragma unroll
        for (int j = 0; j < 5; ++j) out[j] = sel(e.ident, X[j], out[j]);
    }
}

// eigen_leftTransform (euler.cl:434-489) in the interface frame:
//   q = (g-1)(X0 vSq/2 - X_m.v + X4), k = Cs (X0 vn - Xn),
//   w = ((q+k)/(2Cs^2), X0 - 2q/(2Cs^2), Xt1 - X0 vt1, Xt2 - X0 vt2, (q-k)/(2Cs^2))
// evaluated as q = (g-1)(X0 |v|^2/2 + (X4 - X_m.v)), k' = Xn - X0 vn = -k/Cs.
template <typename V>
__device__ __forceinline__ void left(V* w, const Eig<V>& e, const Eos& s, const V* X) {
    V const mv = fma(X[3], e.vt2, fma(X[2], e.vt1, mul(X[1], e.vn)));
    V const q = mul(splat<V>(s.g1), fma(X[0], e.hvSq, sub(X[4], mv)));
    V const kp = fnms(X[0], e.vn, X[1]);
    w[0] = mul(fnms(e.Cs, kp, q), e.invD);
    w[1] = fnms(q, e.invD2, X[0]);
    w[2] = fnms(X[0], e.vt1, X[2]);
    w[3] = fnms(X[0], e.vt2, X[3]);
    w[4] = mul(fma(e.Cs, kp, q), e.invD);
    identLanes(w, e, X);
}

// eigen_rightTransform (euler.cl:493-542) in the interface frame:
//   S = W0 + W1 + W4, D = W4 - W0,
//   F = (S, S vn + Cs D, S vt1 + W2, S vt2 + W3, hT (W0 + W4) + Cs vn D + vSq W1 / 2 + vt1 W2 + vt2 W3)
template <typename V>
__device__ __forceinline__ void right(V* F, const Eig<V>& e, const V* W) {
    V const S = add(add(W[0], W[1]), W[4]);
    V const D = sub(W[4], W[0]);
    V const CsD = mul(e.Cs, D);
    V const f1 = fma(S, e.vn, CsD);
    V const f2 = fma(S, e.vt1, W[2]);
    V const f3 = fma(S, e.vt2, W[3]);
    V f4 = mul(e.hT, add(W[0], W[4]));
    f4 = fma(e.vn, CsD, f4);
    f4 = fma(e.hvSq, W[1], f4);
    f4 = fma(e.vt1, W[2], f4);
    f4 = fma(e.vt2, W[3], f4);
    F[0] = S;
    F[1] = f1;
    F[2] = f2;
    F[3] = f3;
    F[4] = f4;
    identLanes(F, e, W);
}

// Roe flux without a flux limiter (roe.cl:17-163) from the one-sided
// projections: lambda L.(UL+UR)/2 - |lambda| L.(UR-UL)/2 equals
// max(lambda, 0) L.UL + min(lambda, 0) L.UR component by component.
template <typename V>
__device__ __forceinline__ void roeSplit(V* F, const Eos& s, const C5<V>& UL, const C5<V>& UR) {
    Eig<V> e;
    eigen(e, s, UL, UR);
    V wL[5], wR[5], fe[5];
    left(wL, e, s, UL.u);
    left(wR, e, s, UR.u);
    V const zero = splat<V>(0.f);
    V const l0 = sub(e.vn, e.Cs), l4 = add(e.vn, e.Cs);
    V const p0 = vmax(l0, zero), m0 = vmin(l0, zero);
    V const p1 = vmax(e.vn, zero), m1 = vmin(e.vn, zero);
    V const p4 = vmax(l4, zero), m4 = vmin(l4, zero);
    fe[0] = fma(p0, wL[0], mul(m0, wR[0]));
    fe[1] = fma(p1, wL[1], mul(m1, wR[1]));
    fe[2] = fma(p1, wL[2], mul(m1, wR[2]));
    fe[3] = fma(p1, wL[3], mul(m1, wR[3]));
    fe[4] = fma(p4, wL[4], mul(m4, wR[4]));
    right(F, e, fe);
}

// Half slope .5 phi(r) dU of "plm cons" (plm.cl:27-91) for a limiter fixed at
// compile time; the symmetric limiters have a closed form in dUL, dUR (zero
// unless dUL dUR > 0):
//   minmod             the one of dUL, dUR smaller in magnitude
//   monotized central  sign * min(2|dUL|, |dUL + dUR| / 2, 2|dUR|)
//   superbee           sign * max(min(|dUR|, 2|dUL|), min(2|dUR|, |dUL|))
//   van Leer (abs)     2 dUL dUR / (dUL + dUR)
// Other limiters evaluate the reference's selector and table entry per lane.
template <int LIMC>
__device__ __forceinline__ float halfSlope1(float dUL, float dUR, int limRT) {
    float const prod = mul(dUL, dUR);
    float h = 0.f;
    if constexpr (LIMC == 8) {
        h = mul(.5f, fabsf(dUL) < fabsf(dUR) ? dUL : dUR);
    } else if constexpr (LIMC == 17) {
        float const m = vmin(vmin(fabsf(dUL), fabsf(dUR)), mul(.25f, fabsf(add(dUL, dUR))));
        h = dUR < 0.f ? -m : m;
    } else if constexpr (LIMC == 18) {
        float const a = fabsf(dUL), b = fabsf(dUR);
        float const m = vmax(vmin(b, mul(2.f, a)), vmin(mul(2.f, b), a));
        h = mul(.5f, dUR < 0.f ? -m : m);
    } else if constexpr (LIMC == 20) {
        h = mul(prod, rcp(add(dUL, dUR)));
    } else if constexpr (LIMC < 0) {
        // limiter chosen at run time: the closed forms where one exists, so a
        // kernel with the limiter compiled in gives the same bits
        switch (limRT) {
        case 8: return halfSlope1<8>(dUL, dUR, limRT);
        case 17: return halfSlope1<17>(dUL, dUR, limRT);
        case 18: return halfSlope1<18>(dUL, dUR, limRT);
        case 20: return halfSlope1<20>(dUL, dUR, limRT);
        default: return mul(.5f, fast::plmSigmaD<float>(dUL, dUR, limRT));
        }
    } else {
        return mul(.5f, fast::plmSigmaD<float>(dUL, dUR, LIMC));
    }
    return prod > 0.f ? h : 0.f;
}

template <int LIMC>
__device__ __forceinline__ float halfSlope(float dUL, float dUR, int limRT) { return halfSlope1<LIMC>(dUL, dUR, limRT); }

template <int LIMC>
__device__ __forceinline__ float2 halfSlope(float2 dUL, float2 dUR, int limRT) {
    if constexpr (LIMC == 20) {
        float2 const prod = mul(dUL, dUR);
        float2 const h = mul(prod, rcp(add(dUL, dUR)));
        return sel(gt(prod, splat<float2>(0.f)), h, splat<float2>(0.f));
    } else {
        return make_float2(halfSlope1<LIMC>(dUL.x, dUR.x, limRT), halfSlope1<LIMC>(dUL.y, dUR.y, limRT));
    }
}

}  // namespace lanes
}  // namespace hc

namespace hc {
namespace lanes {

// ---- the per-cell epilogue ----------------------------------------------------

// constrainU (euler.cl:697-717): rho >= rhoMin, P >= PMin, through the
// primitive variables and back.
template <typename V>
__device__ __forceinline__ void constrain(V* u, const Eos& s, float invg1) {
    V const rhoMin = splat<V>(s.rhoMin);
    u[0] = vmax(u[0], rhoMin);
    V const inv = rcp(u[0]);
    V const vx = mul(u[1], inv), vy = mul(u[2], inv), vz = mul(u[3], inv);
    V const m2 = fma(u[3], u[3], fma(u[2], u[2], mul(u[1], u[1])));
    V P = sel(lt(u[0], rhoMin), splat<V>(0.f), mul(splat<V>(s.g1), fnms(mul(splat<V>(.5f), m2), inv, u[4])));
    P = vmax(P, splat<V>(s.PMin));
    V const rho = u[0];
    u[1] = mul(vx, rho);
    u[2] = mul(vy, rho);
    u[3] = mul(vz, rho);
    V const vsq = fma(vz, vz, fma(vy, vy, mul(vx, vx)));
    u[4] = fma(P, splat<V>(invg1), mul(rho, mul(splat<V>(.5f), vsq)));
}

// calcDTCell (calcDT.cl:38-73): min over the active sides of
// dx / max(|vn - Cs|, |vn + Cs|, 1e-9), with Cs = 0 where P <= PMin and
// infinite where rho < rhoMin.
template <typename V, int DIM>
__device__ __forceinline__ V dtCell(const V* u, const Eos& s, const float* gdx) {
    V const rhoMin = splat<V>(s.rhoMin), zero = splat<V>(0.f);
    auto const thin = lt(u[0], rhoMin);
    V const inv = rcp(u[0]);
    V const m2 = fma(u[3], u[3], fma(u[2], u[2], mul(u[1], u[1])));
    V const P = sel(thin, zero, mul(splat<V>(s.g1), fnms(mul(splat<V>(.5f), m2), inv, u[4])));
    V Cs = sqr(mul(mul(splat<V>(s.gamma), P), inv));
    Cs = sel(thin, splat<V>(__int_as_float(0x7f800000)), Cs);
    Cs = sel(le(P, splat<V>(s.PMin)), zero, Cs);
    V dt = splat<V>(__int_as_float(0x7f800000));
#pragma unroll
    for (int side = 0; side < DIM; ++side) {
        V const vn = sel(thin, zero, mul(u[1 + side], inv));
        V a = vmax(absv(sub(vn, Cs)), absv(add(vn, Cs)));
        a = vmax(splat<V>(1e-9f), a);
        dt = vmin(dt, mul(splat<V>(gdx[side]), rcp(a)));
    }
    return dt;
}

}  // namespace lanes
}  // namespace hc
