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
__device__ __forceinline__ bool lanesAnd(bool a, bool b) { return a && b; }
__device__ __forceinline__ B2 lanesAnd(B2 a, B2 b) { return {a.x && b.x, a.y && b.y}; }

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

// -x (exact).  Scalar FMAs take a negated operand for free; a register pair
// needs one packed multiply, so the formulas below negate shared operands once
// and use fma(-a, b, c) where c - a b is meant.
__device__ __forceinline__ float neg(float x) { return -x; }
__device__ __forceinline__ float2 neg(float2 x) { return __fmul2_rn(x, make_float2(-1.f, -1.f)); }

// ---- per-lane operations ----------------------------------------------------

// The approximate reciprocal, reciprocal square root and square root as single
// hardware instructions (PTX .approx.ftz): the forms without .ftz add a
// rescaling of subnormal arguments around each.  No argument here is
// subnormal in a valid state (densities >= 1e-5 where a side is not vacuum,
// 2 Cs^2 >= 8e-6 where Cs is not 0, |dUL + dUR| >= 2^-126 wherever the van
// Leer product is positive), and for normal arguments both forms give the
// same value.
__device__ __forceinline__ float rcp(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float rsq(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sqr(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
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
    int hllcMethod;   // euler-hllc's hllcMethod, 0..2
    float invg1;      // 1 / (gamma - 1)
    int recon;        // HC_RECON_*
    float entropyFactor;   // the Roe flux's entropy fix factor, 0: off
};

// A conserved state in the interface frame: rho, m_n, m_t1, m_t2, ETotal.
template <typename V> struct C5 { V u[5]; };

template <typename V> struct Eig {
    V vn, vt1, vt2, hT, Cs;
    V hvSq;          // |v|^2 / 2
    V invD;          // 1 / (2 Cs^2)
    V nCs, nInvD2;   // -Cs, -2 / (2 Cs^2)
    Mask<V> ident;   // rho < rhoMin: the transforms are the identity
};

// The Roe average with both sides above the vacuum threshold
// (euler.cl:347-430): one reciprocal square root per side gives
// sqrt(rho) = rho rs, 1/rho = rs^2 and the Roe weights.
// Also returns the left side's pressure and 1/rho, and the lanes where the
// enthalpy fell below its threshold (hTotal and Cs replaced).
template <typename V>
__device__ __forceinline__ V eigenRoe(Eig<V>& e, const Eos& s, const C5<V>& UL, const C5<V>& UR, V& PLout, V& invLout,
                                      Mask<V>& lowOut) {
    V const half = splat<V>(.5f), nhalf = splat<V>(-.5f), g1 = splat<V>(s.g1), rhoMin = splat<V>(s.rhoMin),
            zero = splat<V>(0.f);
    V const rsL = rsq(UL.u[0]), rsR = rsq(UR.u[0]);
    V const invL = mul(rsL, rsL), invR = mul(rsR, rsR);
    V const sL = mul(UL.u[0], rsL), sR = mul(UR.u[0], rsR);
    V const m2L = fma(UL.u[3], UL.u[3], fma(UL.u[2], UL.u[2], mul(UL.u[1], UL.u[1])));
    V const m2R = fma(UR.u[3], UR.u[3], fma(UR.u[2], UR.u[2], mul(UR.u[1], UR.u[1])));
    V const PL = sel(lt(UL.u[0], rhoMin), zero, mul(g1, fma(mul(nhalf, m2L), invL, UL.u[4])));
    V const PR = sel(lt(UR.u[0], rhoMin), zero, mul(g1, fma(mul(nhalf, m2R), invR, UR.u[4])));
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
    PLout = PL;
    invLout = invL;
    lowOut = low;
    return mul(sL, sR);   // the averaged density
}

template <typename V>
__device__ __forceinline__ V eigenRoe(Eig<V>& e, const Eos& s, const C5<V>& UL, const C5<V>& UR) {
    V PL, invL;
    Mask<V> low;
    return eigenRoe(e, s, UL, UR, PL, invL, low);
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
    e.nInvD2 = mul(splat<V>(-2.f), e.invD);
    e.nCs = neg(e.Cs);
}

__device__ __forceinline__ void eigen(Eig<float>& e, const Eos& s, const C5<float>& UL, const C5<float>& UR) {
    bool const lv = UL.u[0] < 1e-5f, rv = UR.u[0] < 1e-5f;
    float const rho = (lv || rv) ? eigenVac(e, s, UL, UR, lv, rv) : eigenRoe(e, s, UL, UR);
    finishEig(e, s, rho);
}

// A lane pair with a vacuum side in either lane: each lane on its own.  Kept
// out of line: it is rare, and inlined at every interface it would crowd the
// instruction cache.
static __device__ __noinline__ void eigenLanewise(Eig<float2>& e, const Eos& s, const C5<float2>& UL, const C5<float2>& UR) {
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
        setLane(e.nInvD2, k, e1.nInvD2);
        setLane(e.nCs, k, e1.nCs);
        if (k) e.ident.y = e1.ident; else e.ident.x = e1.ident;
    }
}

__device__ __forceinline__ void eigen(Eig<float2>& e, const Eos& s, const C5<float2>& UL, const C5<float2>& UR) {
    B2 const lv = lt(UL.u[0], splat<float2>(1e-5f)), rv = lt(UR.u[0], splat<float2>(1e-5f));
    if (!any(lv || rv)) {
        float2 const rho = eigenRoe(e, s, UL, UR);
        finishEig(e, s, rho);
    } else {
        eigenLanewise(e, s, UL, UR);
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
template <typename V, bool IDENT = true>
__device__ __forceinline__ void left(V* w, const Eig<V>& e, const Eos& s, const V* X) {
    V const mv = fma(X[3], e.vt2, fma(X[2], e.vt1, mul(X[1], e.vn)));
    V const q = mul(splat<V>(s.g1), fma(X[0], e.hvSq, sub(X[4], mv)));
    V const nX0 = neg(X[0]);
    V const kp = fma(nX0, e.vn, X[1]);
    w[0] = mul(fma(e.nCs, kp, q), e.invD);
    w[1] = fma(q, e.nInvD2, X[0]);
    w[2] = fma(nX0, e.vt1, X[2]);
    w[3] = fma(nX0, e.vt2, X[3]);
    w[4] = mul(fma(e.Cs, kp, q), e.invD);
    if constexpr (IDENT) identLanes(w, e, X);
}

// eigen_rightTransform (euler.cl:493-542) in the interface frame:
//   S = W0 + W1 + W4, D = W4 - W0,
//   F = (S, S vn + Cs D, S vt1 + W2, S vt2 + W3, hT (W0 + W4) + Cs vn D + vSq W1 / 2 + vt1 W2 + vt2 W3)
template <typename V, bool IDENT = true>
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
    if constexpr (IDENT) identLanes(F, e, W);
}

// fluxFromCons (euler.cl:271-291) in the interface frame:
// (rho v_n, m_n v_n + P, m_t1 v_n, m_t2 v_n, (ETotal + P) v_n); also v_n and P.
template <typename V>
__device__ __forceinline__ void fluxOf(V* F, V& P, const Eos& s, const C5<V>& U) {
    V const inv = rcp(U.u[0]);
    V const vn = mul(U.u[1], inv);
    V const m2 = fma(U.u[3], U.u[3], fma(U.u[2], U.u[2], mul(U.u[1], U.u[1])));
    P = sel(lt(U.u[0], splat<V>(s.rhoMin)), splat<V>(0.f),
            mul(splat<V>(s.g1), fma(mul(splat<V>(-.5f), m2), inv, U.u[4])));
    F[0] = mul(U.u[0], vn);
    F[1] = fma(U.u[1], vn, P);
    F[2] = mul(U.u[2], vn);
    F[3] = mul(U.u[3], vn);
    F[4] = mul(add(U.u[4], P), vn);
}

// The slowest and fastest waves v_n -/+ Cs of one state (euler.lua:329-337):
// Cs = 0 where P <= PMin, infinite where rho < rhoMin; v_n = 0 where rho < rhoMin.
template <typename V>
__device__ __forceinline__ void wavesOf(V& lmin, V& lmax, const Eos& s, const C5<V>& U, V P) {
    V const inv = rcp(U.u[0]);
    auto const thin = lt(U.u[0], splat<V>(s.rhoMin));
    V Cs = sqr(mul(mul(splat<V>(s.gamma), P), inv));
    Cs = sel(thin, splat<V>(__int_as_float(0x7f800000)), Cs);
    Cs = sel(le(P, splat<V>(s.PMin)), splat<V>(0.f), Cs);
    V const vn = sel(thin, splat<V>(0.f), mul(U.u[1], inv));
    lmin = sub(vn, Cs);
    lmax = add(vn, Cs);
}

// Rusanov flux (hydro/flux/rusanov.cl): .5 (FL + FR - lambda (UR - UL)) with
// lambda = max(|v_n - Cs|, |v_n + Cs|) of the right state (the reference's
// loop over the two sides keeps the last one's bound).
template <typename V>
__device__ __forceinline__ void rusanov(V* F, const Eos& s, const C5<V>& UL, const C5<V>& UR) {
    V FL[5], FR[5], PL, PR, lmin, lmax;
    fluxOf(FL, PL, s, UL);
    fluxOf(FR, PR, s, UR);
    wavesOf(lmin, lmax, s, UR, PR);
    V const nlam = neg(vmax(absv(lmin), absv(lmax)));
    V const half = splat<V>(.5f);
#pragma unroll
    for (int j = 0; j < 5; ++j) F[j] = mul(half, fma(nlam, sub(UR.u[j], UL.u[j]), add(FL[j], FR[j])));
}

// HLL flux (hydro/flux/hll.cl, waves 'Davis direct bounded'): sL = min(v_n - Cs
// of UL, Roe-average v_n - Cs), sR = max(v_n + Cs of UR, Roe-average v_n + Cs);
// FL where 0 <= sL, FR where sR <= 0, else
// (sR FL - sL FR + sL sR (UR - UL)) / (sR - sL).
template <typename V>
__device__ __forceinline__ void hll(V* F, const Eos& s, const C5<V>& UL, const C5<V>& UR) {
    Eig<V> e;
    eigen(e, s, UL, UR);
    V FL[5], FR[5], PL, PR, lminL, lmaxL, lminR, lmaxR;
    fluxOf(FL, PL, s, UL);
    fluxOf(FR, PR, s, UR);
    wavesOf(lminL, lmaxL, s, UL, PL);
    wavesOf(lminR, lmaxR, s, UR, PR);
    V const sL = vmin(lminL, sub(e.vn, e.Cs));
    V const sR = vmax(lmaxR, add(e.vn, e.Cs));
    V const inv = rcp(sub(sR, sL));
    V const sLsR = mul(sL, sR);
    V const nsL = neg(sL);
    V const zero = splat<V>(0.f);
    auto const left = le(zero, sL), right = le(sR, zero);
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        V const mid = mul(fma(sLsR, sub(UR.u[j], UL.u[j]), fma(nsL, FR[j], mul(sR, FL[j]))), inv);
        F[j] = sel(left, FL[j], sel(right, FR[j], mid));
    }
}

// |lambda| of a Roe wave after useEntropyFluxFix (roe.cl:83-101): where
// |lambda| < dws = factor Cs, |sign(lambda) (lambda^2 / dws + dws) / 2|, with
// OpenCL's sign(0) = 0 keeping a zero speed zero; |lambda| itself with the
// fix off (factor 0: nothing is below dws = 0).
template <typename V>
__device__ __forceinline__ V fixedAbs(V lambda, V Cs, float factor) {
    V const a = absv(lambda), zero = splat<V>(0.f);
    V const dws = mul(splat<V>(factor), Cs);
    V const fixd = mul(splat<V>(.5f), add(mul(mul(lambda, lambda), rcp(dws)), dws));
    return sel(lt(a, dws), sel(le(a, zero), zero, fixd), a);
}

// Roe flux without a flux limiter (roe.cl:17-163) in the fluxFromCons form
// Euler inherits (roeUseFluxFromCons, eqn.lua:46):
//   F = (F(UL) + F(UR)) / 2 - R |Lambda| L.(UR - UL) / 2
// (|Lambda| after the entropy fix where it is on).
template <typename V>
__device__ __forceinline__ void roeCentral(V* F, const Eos& s, const C5<V>& UL, const C5<V>& UR) {
    Eig<V> e;
    eigen(e, s, UL, UR);
    V dU[5], dW[5], fe[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) dU[j] = sub(UR.u[j], UL.u[j]);
    left(dW, e, s, dU);
    V const nh = splat<V>(-.5f);
    V const c0 = mul(nh, fixedAbs(sub(e.vn, e.Cs), e.Cs, s.entropyFactor));
    V const c1 = mul(nh, fixedAbs(e.vn, e.Cs, s.entropyFactor));
    V const c4 = mul(nh, fixedAbs(add(e.vn, e.Cs), e.Cs, s.entropyFactor));
    fe[0] = mul(c0, dW[0]);
    fe[1] = mul(c1, dW[1]);
    fe[2] = mul(c1, dW[2]);
    fe[3] = mul(c1, dW[3]);
    fe[4] = mul(c4, dW[4]);
    right(F, e, fe);
    V FL[5], FR[5], PL, PR;
    fluxOf(FL, PL, s, UL);
    fluxOf(FR, PR, s, UR);
    V const half = splat<V>(.5f);
#pragma unroll
    for (int j = 0; j < 5; ++j) F[j] = fma(half, add(FL[j], FR[j]), F[j]);
}

// With the plain Roe average (both densities above the vacuum threshold,
// the enthalpy above its floor, the averaged density at least rhoMin) the
// Roe matrix has property U, F(UR) - F(UL) = R Lambda L.(UR - UL), and the
// flux above equals the upwind form F(UL) + R min(Lambda, 0) L.(UR - UL):
// one physical flux instead of two, built from the left side's pressure and
// 1/rho that the average already has.  Other states, and every state with the
// entropy fix on (it changes |Lambda| but not Lambda), take the form above.
template <typename V>
__device__ __forceinline__ void roe(V* F, const Eos& s, const C5<V>& UL, const C5<V>& UR) {
    if constexpr (nlanes<V>() == 1) {
        bool const lv = UL.u[0] < 1e-5f, rv = UR.u[0] < 1e-5f;
        Eig<float> e;
        float PL = 0.f, invL = 0.f;
        bool low = false;
        float const rho = (lv || rv) ? eigenVac(e, s, UL, UR, lv, rv) : eigenRoe(e, s, UL, UR, PL, invL, low);
        finishEig(e, s, rho);
        bool const pu = !(lv || rv || low || e.ident) && s.entropyFactor == 0.f;
        float dU[5], dW[5], fe[5];
#pragma unroll
        for (int j = 0; j < 5; ++j) dU[j] = sub(UR.u[j], UL.u[j]);
        left(dW, e, s, dU);
        float const l0 = sub(e.vn, e.Cs), l4 = add(e.vn, e.Cs);
        float const c0 = pu ? vmin(l0, 0.f) : mul(-.5f, fixedAbs(l0, e.Cs, s.entropyFactor));
        float const c1 = pu ? vmin(e.vn, 0.f) : mul(-.5f, fixedAbs(e.vn, e.Cs, s.entropyFactor));
        float const c4 = pu ? vmin(l4, 0.f) : mul(-.5f, fixedAbs(l4, e.Cs, s.entropyFactor));
        fe[0] = mul(c0, dW[0]);
        fe[1] = mul(c1, dW[1]);
        fe[2] = mul(c1, dW[2]);
        fe[3] = mul(c1, dW[3]);
        fe[4] = mul(c4, dW[4]);
        right(F, e, fe);
        if (pu) {
            float const vn = mul(UL.u[1], invL);
            F[0] = add(F[0], UL.u[1]);
            F[1] = add(F[1], fma(UL.u[1], vn, PL));
            F[2] = fma(UL.u[2], vn, F[2]);
            F[3] = fma(UL.u[3], vn, F[3]);
            F[4] = fma(add(UL.u[4], PL), vn, F[4]);
        } else {
            float FL[5], FR[5], PLc, PRc;
            fluxOf(FL, PLc, s, UL);
            fluxOf(FR, PRc, s, UR);
#pragma unroll
            for (int j = 0; j < 5; ++j) F[j] = fma(.5f, add(FL[j], FR[j]), F[j]);
        }
    } else {
        roeCentral<V>(F, s, UL, UR);
    }
}

// The Roe flux of one interface (V = float) or two at once on register pairs
// (V = float2, roeUp2), in the upwind form F(UL) + R min(Lambda, 0)
// L.(UR - UL), operation for operation as roe<float> evaluates it where the
// Roe average is the plain one.  Returns whether every lane has the plain
// average (no vacuum side, enthalpy above its floor, averaged density at
// least rhoMin) and the entropy fix is off; where a lane has not, F is not
// that lane's flux and the caller evaluates roe<float> for it.
template <typename V>
__device__ __forceinline__ bool roeUp(V* F, const Eos& s, const C5<V>& UL, const C5<V>& UR) {
    if (s.entropyFactor != 0.f) return false;   // the entropy fix: roe<float> evaluates every face
    Mask<V> const lv = lt(UL.u[0], splat<V>(1e-5f)), rv = lt(UR.u[0], splat<V>(1e-5f));
    Eig<V> e;
    V PL, invL;
    Mask<V> low;
    V const rho = eigenRoe(e, s, UL, UR, PL, invL, low);
    finishEig(e, s, rho);
    V dU[5], dW[5], fe[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) dU[j] = sub(UR.u[j], UL.u[j]);
    left<V, false>(dW, e, s, dU);   // an identity lane is not plain: no lane select
    V const zero = splat<V>(0.f);
    V const c0 = vmin(sub(e.vn, e.Cs), zero);
    V const c1 = vmin(e.vn, zero);
    V const c4 = vmin(add(e.vn, e.Cs), zero);
    fe[0] = mul(c0, dW[0]);
    fe[1] = mul(c1, dW[1]);
    fe[2] = mul(c1, dW[2]);
    fe[3] = mul(c1, dW[3]);
    fe[4] = mul(c4, dW[4]);
    right<V, false>(F, e, fe);
    V const vn = mul(UL.u[1], invL);
    F[0] = add(F[0], UL.u[1]);
    F[1] = add(F[1], fma(UL.u[1], vn, PL));
    F[2] = fma(UL.u[2], vn, F[2]);
    F[3] = fma(UL.u[3], vn, F[3]);
    F[4] = fma(add(UL.u[4], PL), vn, F[4]);
    return !any(lv || rv || low || e.ident);
}

__device__ __forceinline__ bool roeUp2(float2* F, const Eos& s, const C5<float2>& UL, const C5<float2>& UR) {
    return roeUp<float2>(F, s, UL, UR);
}

// HLLC flux (hydro/flux/euler-hllc.cl, 2012 Toro; waves as hll) in the
// interface frame.  The star state of side K (speed sK):
//   method 0: F = FK + sK (UK* - UK), rho* = rho (sK - vn) / (sK - s*),
//             m* = rho* (s*, vt1, vt2), E* = rho* (E / rho + (s* - vn)(s* + P / (rho (sK - vn))))
//   method 1: F = (s* (sK U - FK) + sK (P + rho (sK - vn)(s* - vn)) (0, 1, 0, 0, s*)) / (sK - s*)
//   method 2: as method 1 with P + rho (sK - vn)(s* - vn) replaced by the
//             average PLR of the two sides
// chosen, lane by lane, in the reference's order: FL where 0 <= sL, the left
// star where sL <= 0 <= s*, the right star where s* <= 0 <= sR, FR where
// sR <= 0, else the HLL average.
template <typename V>
__device__ __forceinline__ void hllc(V* F, const Eos& s, const C5<V>& UL, const C5<V>& UR) {
    Eig<V> e;
    eigen(e, s, UL, UR);
    V FL[5], FR[5], PL, PR, lminL, lmaxL, lminR, lmaxR;
    fluxOf(FL, PL, s, UL);
    fluxOf(FR, PR, s, UR);
    wavesOf(lminL, lmaxL, s, UL, PL);
    wavesOf(lminR, lmaxR, s, UR, PR);
    V const sL = vmin(lminL, sub(e.vn, e.Cs));
    V const sR = vmax(lmaxR, add(e.vn, e.Cs));
    V const vnL = mul(UL.u[1], rcp(UL.u[0])), vnR = mul(UR.u[1], rcp(UR.u[0]));
    V const aL = sub(sL, vnL), aR = sub(sR, vnR);   // sK - vn
    V const rhoaL = mul(UL.u[0], aL), rhoaR = mul(UR.u[0], aR);
    // s* = (rhoR vnR aR - rhoL vnL aL + PL - PR) / (rhoR aR - rhoL aL)
    V const sStar = mul(sub(add(fma(rhoaR, vnR, neg(mul(rhoaL, vnL))), PL), PR), rcp(sub(rhoaR, rhoaL)));
    V SL[5], SR[5];
    auto star = [&](V* S, const C5<V>& U, const V* FK, V P, V sK, V a, V rhoa) {
        V const d = rcp(sub(sK, sStar));
        if (s.hllcMethod == 0) {
            V const rs = mul(mul(U.u[0], a), d);
            V const us[5] = {rs, mul(rs, sStar), mul(rs, mul(U.u[2], rcp(U.u[0]))), mul(rs, mul(U.u[3], rcp(U.u[0]))),
                             mul(rs, fma(sub(sStar, sub(sK, a)), add(sStar, mul(P, rcp(rhoa))), mul(U.u[4], rcp(U.u[0]))))};
#pragma unroll
            for (int j = 0; j < 5; ++j) S[j] = fma(sK, sub(us[j], U.u[j]), FK[j]);
        } else {
            V const vn = sub(sK, a);
            V const Pk = s.hllcMethod == 1
                ? fma(rhoa, sub(sStar, vn), P)
                : mul(splat<V>(.5f), add(add(add(PL, PR), mul(rhoaL, sub(sStar, vnL))), mul(rhoaR, sub(sStar, vnR))));
#pragma unroll
            for (int j = 0; j < 5; ++j) S[j] = mul(sStar, sub(mul(sK, U.u[j]), FK[j]));
            S[1] = fma(sK, Pk, S[1]);
            S[4] = fma(mul(sK, Pk), sStar, S[4]);
#pragma unroll
            for (int j = 0; j < 5; ++j) S[j] = mul(S[j], d);
        }
    };
    star(SL, UL, FL, PL, sL, aL, rhoaL);
    star(SR, UR, FR, PR, sR, aR, rhoaR);
    V const zero = splat<V>(0.f);
    V const inv = rcp(sub(sR, sL));
    V const sLsR = mul(sL, sR);
    V const nsL = neg(sL);
    auto const c0 = le(zero, sL), c3 = le(sR, zero);
    auto const c1 = le(sL, zero);
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        V const avg = mul(fma(sLsR, sub(UR.u[j], UL.u[j]), fma(nsL, FR[j], mul(sR, FL[j]))), inv);
        V r = avg;
        r = sel(c3, FR[j], r);
        r = sel(lanesAnd(le(sStar, zero), le(zero, sR)), SR[j], r);
        r = sel(lanesAnd(c1, le(zero, sStar)), SL[j], r);
        r = sel(c0, FL[j], r);
        F[j] = r;
    }
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

// ---- "plm prim" and "plm athena" ---------------------------------------------

// primFromCons (euler.cl:140-159) in the interface frame: rho, v_n, v_t1, v_t2, P.
template <typename V>
__device__ __forceinline__ void primOf(V* w, const Eos& s, const C5<V>& U) {
    V const inv = rcp(U.u[0]);
    V const m2 = fma(U.u[3], U.u[3], fma(U.u[2], U.u[2], mul(U.u[1], U.u[1])));
    w[0] = U.u[0];
    w[1] = mul(U.u[1], inv);
    w[2] = mul(U.u[2], inv);
    w[3] = mul(U.u[3], inv);
    w[4] = sel(lt(U.u[0], splat<V>(s.rhoMin)), splat<V>(0.f),
               mul(splat<V>(s.g1), fma(mul(splat<V>(-.5f), m2), inv, U.u[4])));
}

// consFromPrim (euler.cl:163-173) in the interface frame.
template <typename V>
__device__ __forceinline__ void consOf(C5<V>& U, const Eos& s, const V* w) {
    U.u[0] = w[0];
    U.u[1] = mul(w[1], w[0]);
    U.u[2] = mul(w[2], w[0]);
    U.u[3] = mul(w[3], w[0]);
    V const vsq = fma(w[3], w[3], fma(w[2], w[2], mul(w[1], w[1])));
    U.u[4] = fma(w[4], splat<V>(s.invg1), mul(w[0], mul(splat<V>(.5f), vsq)));
}

// "plm prim"'s half slope .5 phi(r) dWR with r = dWL / dWR (0 where dWR = 0),
// from the reference's limiter table (plm.cl:223-231).
__device__ __forceinline__ float halfSlopePrim(float dWL, float dWR, int lim) {
    float const r = dWR == 0.f ? 0.f : __fdiv_rn(dWL, dWR);
    return mul(.5f, mul(fast::limiter<float>(lim, r), dWR));
}
__device__ __forceinline__ float2 halfSlopePrim(float2 dWL, float2 dWR, int lim) {
    return make_float2(halfSlopePrim(dWL.x, dWR.x, lim), halfSlopePrim(dWL.y, dWR.y, lim));
}

// "plm prim" (plm.cl:191-253): the cell's L and R states from its own and
// its neighbours' primitives.
template <typename V>
__device__ __forceinline__ void plmPrim(C5<V>& L, C5<V>& R, const Eos& s, const V* Wm, const V* W0, const V* Wp,
                                        int lim) {
    V nL[5], nR[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        V const h = halfSlopePrim(sub(W0[j], Wm[j]), sub(Wp[j], W0[j]), lim);
        nL[j] = sub(W0[j], h);
        nR[j] = add(W0[j], h);
    }
    consOf(L, s, nL);
    consOf(R, s, nR);
}

// "plm athena" (plm.cl:782-879): the primitive differences projected on the
// eigenvectors at the cell (eigen_forCell, euler.cl:315-342), limited per
// wave (zero unless the left and right projections agree in sign, else
// sign(c) min(2 min(|l|, |r|), min(|c|, |g|)) with the central and the
// harmonic differences c and g), projected back, clamped into the range of
// the neighbouring primitives; L is built from the right-edge value and R
// from the left-edge value, as plm.cl:877-878 assigns them.
template <typename V>
__device__ __forceinline__ void plmAthena(C5<V>& L, C5<V>& R, const Eos& s, const C5<V>& U0, const V* Wm,
                                          const V* W0, const V* Wp) {
    V const zero = splat<V>(0.f), half = splat<V>(.5f), two = splat<V>(2.f);
    Eig<V> e;
    e.vn = W0[1];
    e.vt1 = W0[2];
    e.vt2 = W0[3];
    e.hvSq = mul(half, fma(W0[3], W0[3], fma(W0[2], W0[2], mul(W0[1], W0[1]))));
    e.hT = mul(add(W0[4], U0.u[4]), rcp(W0[0]));
    e.Cs = sqr(mul(splat<V>(s.g1), sub(e.hT, e.hvSq)));
    finishEig(e, s, W0[0]);
    V dWL[5], dWR[5], dWC[5], dWG[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        dWL[j] = sub(W0[j], Wm[j]);
        dWR[j] = sub(Wp[j], W0[j]);
        dWC[j] = mul(half, sub(Wp[j], Wm[j]));
        V const g = mul(mul(mul(two, dWL[j]), dWR[j]), rcp(add(dWL[j], dWR[j])));
        dWG[j] = sel(le(mul(dWL[j], dWR[j]), zero), zero, g);
    }
    V dal[5], dar[5], dac[5], dag[5];
    left(dal, e, s, dWL);
    left(dar, e, s, dWR);
    left(dac, e, s, dWC);
    left(dag, e, s, dWG);
    V da[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        V const m = vmin(mul(two, vmin(absv(dal[j]), absv(dar[j]))), vmin(absv(dac[j]), absv(dag[j])));
        V const sm = sel(gt(dac[j], zero), m, sel(lt(dac[j], zero), neg(m), zero));
        da[j] = sel(gt(mul(dal[j], dar[j]), zero), sm, zero);
    }
    V dWm[5];
    right(dWm, e, da);
    V lv[5], rv[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        V l = fnms(half, dWm[j], W0[j]);
        V r = fma(half, dWm[j], W0[j]);
        V const C = add(r, l);
        l = vmax(vmin(W0[j], Wm[j]), l);
        l = vmin(vmax(W0[j], Wm[j]), l);
        r = sub(C, l);
        r = vmax(vmin(W0[j], Wp[j]), r);
        r = vmin(vmax(W0[j], Wp[j]), r);
        l = sub(C, r);
        lv[j] = l;
        rv[j] = r;
    }
    consOf(L, s, rv);
    consOf(R, s, lv);
}

}  // namespace lanes
}  // namespace hc

namespace hc {
namespace lanes {

// ---- the per-cell epilogue ----------------------------------------------------

// constrainU (euler.cl:697-717): rho >= rhoMin, P >= PMin, through the
// primitive variables and back.  A cell that needs neither clamp keeps its
// state: the round trip is the identity in exact arithmetic, and in FP32 it
// is not (P (1/(g-1)) with both factors rounded adds 1.5e-8 of the internal
// energy per stage at g = 1.4, a drift of the total energy).
template <typename V>
__device__ __forceinline__ void constrain(V* u, const Eos& s, float invg1) {
    V const rhoMin = splat<V>(s.rhoMin);
    auto const thin = lt(u[0], rhoMin);
    V const rho = vmax(u[0], rhoMin);
    V const inv = rcp(rho);
    V const m2 = fma(u[3], u[3], fma(u[2], u[2], mul(u[1], u[1])));
    V const P0 = mul(splat<V>(s.g1), fma(mul(splat<V>(-.5f), m2), inv, u[4]));
    auto const low = lt(P0, splat<V>(s.PMin));
    if (!any(thin || low)) return;
    V const vx = mul(u[1], inv), vy = mul(u[2], inv), vz = mul(u[3], inv);
    V const P = vmax(P0, splat<V>(s.PMin));
    V const vsq = fma(vz, vz, fma(vy, vy, mul(vx, vx)));
    auto const fix = thin || low;
    u[0] = rho;
    u[1] = sel(fix, mul(vx, rho), u[1]);
    u[2] = sel(fix, mul(vy, rho), u[2]);
    u[3] = sel(fix, mul(vz, rho), u[3]);
    u[4] = sel(fix, fma(P, splat<V>(invg1), mul(rho, mul(splat<V>(.5f), vsq))), u[4]);
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
    V const P = sel(thin, zero, mul(splat<V>(s.g1), fma(mul(splat<V>(-.5f), m2), inv, u[4])));
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
