// hc_fast_math.cuh -- the same Euler / Roe / PLM arithmetic as hc_ref_math.cuh,
// restated in the frame of the interface normal for throughput.
//
// With hydro-cl-lua's Cartesian side-permutation normals
// (hydro/coord/coord.lua:2341-2409) the reference's 5x5 left/right eigenvector
// transforms (hydro/eqn/euler.cl:434-542) contain only 0/1 normal components.
// Expressed in the rotated frame (n, t1, t2) = (side, side+1, side+2) they
// reduce to a handful of shared sub-expressions:
//
//   L.X:  q = (g-1)(X0 vSq/2 - X_m.v + X4),  k = Cs (X0 vn - Xn),
//         w0 = (q + k)/(2Cs^2), w1 = X0 - 2q/(2Cs^2), w2 = Xt1 - X0 vt1,
//         w3 = Xt2 - X0 vt2,   w4 = (q - k)/(2Cs^2)
//   R.W:  S = W0 + W1 + W4,  D = W4 - W0
//         F = (S, S vn + Cs D, S vt1 + W2, S vt2 + W3,
//              hT (W0 + W4) + Cs vn D + vSq W1/2 + vt1 W2 + vt2 W3)
//
// which is algebraically identical to the reference; only rounding differs.
// Branches (vacuum states, rhoMin / PMin guards, the limiter selectors) are
// kept exactly.  Single precision uses the fast reciprocal / square-root
// intrinsics; the FP32 form is held to the density L1 tolerance against the
// FP64 oracle, not to bitwise parity.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace hc {
namespace fast {

template <typename T> struct M;
// FP32: the hardware approximations as single instructions (PTX .approx.ftz;
// the forms without .ftz rescale subnormal arguments around each).  For
// normal arguments and results both forms give the same value.
template <> struct M<float> {
    static __device__ __forceinline__ float rsqrt_(float x) {
        float r;
        asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
        return r;
    }
    static __device__ __forceinline__ float abs_(float x) { return fabsf(x); }
    static __device__ __forceinline__ bool finite_(float x) { return (__float_as_uint(x) & 0x7f800000u) != 0x7f800000u; }
    static __device__ __forceinline__ float rcp(float x) {
        float r;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
        return r;
    }
    static __device__ __forceinline__ float div(float a, float b) {
        float r;
        asm("div.approx.ftz.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
        return r;
    }
    static __device__ __forceinline__ float sqrt_(float x) {
        float r;
        asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
        return r;
    }
    static __device__ __forceinline__ float inf() { return __int_as_float(0x7f800000); }
};
template <> struct M<double> {
    static __device__ __forceinline__ double rsqrt_(double x) { return 1. / sqrt(x); }
    static __device__ __forceinline__ double abs_(double x) { return fabs(x); }
    static __device__ __forceinline__ bool finite_(double x) { return isfinite(x); }
    static __device__ __forceinline__ double rcp(double x) { return 1. / x; }
    static __device__ __forceinline__ double div(double a, double b) { return a / b; }
    static __device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
    static __device__ __forceinline__ double inf() { return __longlong_as_double(0x7ff0000000000000ll); }
};

template <typename T> __device__ __forceinline__ T tmax(T x, T y) { return x < y ? y : x; }
template <typename T> __device__ __forceinline__ T tmin(T x, T y) { return y < x ? y : x; }

// hydro/app.lua:614-635
template <typename T>
__device__ __forceinline__ T limiter(int which, T r) {
    T const z = T(0), one = T(1), two = T(2);
    switch (which) {
    case 0: return z;
    case 1: return one;
    case 2: return r;
    case 3: return T(.5) * (one + r);
    case 4: return M<T>::div(tmax(z, r) * (T(3) * r + one), (r + one) * (r + one));
    case 5: return tmax(z, M<T>::div(T(1.5) * (r + M<T>::abs_(r)), r + two));
    case 6: return tmax(z, M<T>::div(two * (r + M<T>::abs_(r)), r + T(3)));
    case 7: return tmax(z, tmin(two * r, tmin(M<T>::div(one + two * r, T(3)), two)));
    case 8: return tmax(z, tmin(r, one));
    case 9: return tmax(z, tmin(r, T(1.5)));
    case 10: return M<T>::div(T(.5) * (r * r + r), r * r + r + one);
    case 11: return tmax(z, tmin(two * r, tmin(T(.25) + T(.75) * r, T(4))));
    case 12: return tmax(z, tmax(tmin(T(1.5) * r, one), tmin(r, T(1.5))));
    case 13: return tmax(z, tmin(tmin(two * r, T(.75) + T(.25) * r), tmin(T(.25) + T(.75) * r, two)));
    case 14: return M<T>::div(r * r + r, r * r + one);
    case 15: return M<T>::div(two * r, r * r + one);
    case 16: return M<T>::div(tmax(z, r) * two, one + r);
    case 17: return tmax(z, tmin(two, tmin(T(.5) * (one + r), two * r)));
    case 18: return tmax(z, tmax(tmin(one, two * r), tmin(two, r)));
    case 19: return T(.5) * (r + one) * tmin(one, tmin(M<T>::div(T(4) * r, r + one), M<T>::div(T(4), r + one)));
    case 20: return M<T>::div(r + M<T>::abs_(r), one + M<T>::abs_(r));
    }
    return z;
}

template <typename T> struct Eos {
    T gamma, g1, rhoMin, PMin;
    int fluxLimiter, slopeLimiter;
    int hllcMethod;
    T entropyFactor;   // the Roe flux's entropy fix factor, 0: off
};

// A conserved state in the interface frame: rho, m_n, m_t1, m_t2, ETotal.
template <typename T> struct C5 { T u[5]; };

// Roe eigen-state in the interface frame.  ident: the transforms are the
// identity (eig.rho < rhoMin).
template <typename T> struct EigF {
    T vn, vt1, vt2, hT, Cs, vSq, invD;
    bool ident;
};

// Primitive quantities used by the Roe average (euler.cl:140-159, 79-83).
template <typename T>
__device__ __forceinline__ void primOf(const C5<T>& U, const Eos<T>& s, T& inv, T& P) {
    inv = M<T>::rcp(U.u[0]);
    T const m2 = U.u[1] * U.u[1] + U.u[2] * U.u[2] + U.u[3] * U.u[3];
    T const EKin = U.u[0] < s.rhoMin ? T(0) : T(.5) * m2 * inv;
    P = U.u[0] < s.rhoMin ? T(0) : s.g1 * (U.u[4] - EKin);
}

// eigen_forInterface (euler.cl:347-430) in the interface frame.
template <typename T>
__device__ __forceinline__ void eigen(EigF<T>& e, const Eos<T>& s, const C5<T>& UL, const C5<T>& UR) {
    T const eps = T(1e-5);
    bool const lv = UL.u[0] < eps, rv = UR.u[0] < eps;
    T rho;
    if (lv && rv) {
        rho = T(0);
        e.vn = e.vt1 = e.vt2 = T(0);
        e.vSq = T(0);
        e.hT = T(0);
        e.Cs = T(0);
    } else if (lv || rv) {
        const C5<T>& Uo = lv ? UR : UL;
        T inv, P;
        primOf(Uo, s, inv, P);
        rho = Uo.u[0];
        e.vn = Uo.u[1] * inv;
        e.vt1 = Uo.u[2] * inv;
        e.vt2 = Uo.u[3] * inv;
        e.vSq = e.vn * e.vn + e.vt1 * e.vt1 + e.vt2 * e.vt2;
        e.hT = (P + Uo.u[4]) * inv;
        e.Cs = P <= s.PMin ? T(0) : (Uo.u[0] < s.rhoMin ? M<T>::inf() : M<T>::sqrt_(s.gamma * P * inv));
    } else {
        // one reciprocal square root per side gives sqrt(rho) = rho rs,
        // 1/rho = rs^2, and the Roe weights: sqrt(rho) v = m rs,
        // sqrt(rho) hTotal = (P + ETotal) rs
        T const rsL = M<T>::rsqrt_(UL.u[0]), rsR = M<T>::rsqrt_(UR.u[0]);
        T const invL = rsL * rsL, invR = rsR * rsR;
        T const sL = UL.u[0] * rsL, sR = UR.u[0] * rsR;
        T const m2L = UL.u[1] * UL.u[1] + UL.u[2] * UL.u[2] + UL.u[3] * UL.u[3];
        T const m2R = UR.u[1] * UR.u[1] + UR.u[2] * UR.u[2] + UR.u[3] * UR.u[3];
        T const PL = UL.u[0] < s.rhoMin ? T(0) : s.g1 * (UL.u[4] - T(.5) * m2L * invL);
        T const PR = UR.u[0] < s.rhoMin ? T(0) : s.g1 * (UR.u[4] - T(.5) * m2R * invR);
        T const invDen = M<T>::rcp(sL + sR);
        rho = sL * sR;
        e.vn = (UL.u[1] * rsL + UR.u[1] * rsR) * invDen;
        e.vt1 = (UL.u[2] * rsL + UR.u[2] * rsR) * invDen;
        e.vt2 = (UL.u[3] * rsL + UR.u[3] * rsR) * invDen;
        T const hT = ((PL + UL.u[4]) * rsL + (PR + UR.u[4]) * rsR) * invDen;
        e.vSq = e.vn * e.vn + e.vt1 * e.vt1 + e.vt2 * e.vt2;
        T const eKin = T(.5) * e.vSq;
        T const h = hT - eKin;
        if (h < eps) {
            e.hT = eKin;
            e.Cs = T(0);
        } else {
            e.hT = hT;
            e.Cs = M<T>::sqrt_(s.g1 * h);
        }
    }
    e.ident = rho < s.rhoMin;
    e.invD = M<T>::rcp(T(2) * e.Cs * e.Cs);
}

// eigen_leftTransform (euler.cl:434-489) in the interface frame.
template <typename T>
__device__ __forceinline__ void left(T* w, const EigF<T>& e, const Eos<T>& s, const T* X) {
    if (e.ident) {
        for (int j = 0; j < 5; ++j) w[j] = X[j];
        return;
    }
    T const mv = X[1] * e.vn + X[2] * e.vt1 + X[3] * e.vt2;
    T const q = s.g1 * (T(.5) * X[0] * e.vSq - mv + X[4]);
    T const k = e.Cs * (X[0] * e.vn - X[1]);
    w[0] = (q + k) * e.invD;
    w[1] = X[0] - T(2) * q * e.invD;
    w[2] = X[2] - X[0] * e.vt1;
    w[3] = X[3] - X[0] * e.vt2;
    w[4] = (q - k) * e.invD;
}

// eigen_rightTransform (euler.cl:493-542) in the interface frame.
template <typename T>
__device__ __forceinline__ void right(T* F, const EigF<T>& e, const T* W) {
    if (e.ident) {
        for (int j = 0; j < 5; ++j) F[j] = W[j];
        return;
    }
    T const S = W[0] + W[1] + W[4];
    T const D = W[4] - W[0];
    T const CsD = e.Cs * D;
    F[0] = S;
    F[1] = S * e.vn + CsD;
    F[2] = S * e.vt1 + W[2];
    F[3] = S * e.vt2 + W[3];
    F[4] = e.hT * (W[0] + W[4]) + e.vn * CsD + T(.5) * e.vSq * W[1] + e.vt1 * W[2] + e.vt2 * W[3];
}

// Interface data reused by the flux limiter of the neighbouring interfaces.
template <typename T> struct IfaceF {
    EigF<T> e;
    T dW[5];
};

template <typename T>
__device__ __forceinline__ void makeIface(IfaceF<T>& I, const Eos<T>& s, const C5<T>& UL, const C5<T>& UR) {
    eigen(I.e, s, UL, UR);
    T dU[5];
    for (int j = 0; j < 5; ++j) dU[j] = UR.u[j] - UL.u[j];
    left(I.dW, I.e, s, dU);
}

// fluxFromCons (euler.cl:271-291) in the interface frame:
// (rho v_n, m_n v_n + P, m_t1 v_n, m_t2 v_n, (ETotal + P) v_n).
template <typename T>
__device__ __forceinline__ void fluxOf(T* F, const Eos<T>& s, const C5<T>& U) {
    T inv, P;
    primOf(U, s, inv, P);
    T const vn = U.u[1] * inv;
    F[0] = U.u[0] * vn;
    F[1] = U.u[1] * vn + P;
    F[2] = U.u[2] * vn;
    F[3] = U.u[3] * vn;
    F[4] = (U.u[4] + P) * vn;
}

// Roe flux with the flux limiter (roe.cl:17-163, in the fluxFromCons form
// Euler inherits, eqn.lua:46) at interface C; IL / IR are the neighbouring
// interfaces:  F = R.fe + (F(UL) + F(UR)) / 2,
// fe_j = -lambda_j dW_j (sgn + phi (lambda_j dt/dx - sgn)) / 2.
template <typename T>
__device__ __forceinline__ void roeLimited(T* F, const Eos<T>& s, const C5<T>& UL, const C5<T>& UR,
                                           const IfaceF<T>& C, const IfaceF<T>& IL, const IfaceF<T>& IR, T dt_dx) {
    T fe[5];
    T const vn = C.e.vn, Cs = C.e.Cs;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        T lambda = j == 0 ? vn - Cs : (j == 4 ? vn + Cs : vn);
        if (s.entropyFactor != T(0)) {
            // useEntropyFluxFix (roe.cl:83-101)
            T const dws = s.entropyFactor * Cs;
            if (M<T>::abs_(lambda) < dws)
                lambda = (lambda > T(0) ? T(1) : (lambda < T(0) ? T(-1) : lambda)) * T(.5) *
                         (M<T>::div(lambda * lambda, dws) + dws);
        }
        T const sgn = lambda >= T(0) ? T(1) : T(-1);
        T rEig;
        if (C.dW[j] == T(0)) rEig = T(0);
        else rEig = M<T>::div(lambda >= T(0) ? IL.dW[j] : IR.dW[j], C.dW[j]);
        T const phi = limiter<T>(s.fluxLimiter, rEig);
        fe[j] = T(-.5) * lambda * C.dW[j] * (sgn + phi * (lambda * dt_dx - sgn));
    }
    right(F, C.e, fe);
    T FL[5], FR[5];
    fluxOf(FL, s, UL);
    fluxOf(FR, s, UR);
#pragma unroll
    for (int j = 0; j < 5; ++j) F[j] = F[j] + T(.5) * (FL[j] + FR[j]);
}

// "plm cons" slope of one component: returns sigma.
template <typename T>
__device__ __forceinline__ T plmSigmaD(T dUL, T dUR, int lim) {
    T const dUC = T(.5) * (dUR - dUL);
    bool const pos = dUC >= T(0);
    T const num = pos ? dUL : dUR;
    T const den = pos ? dUR : dUL;
    T const r = den == T(0) ? T(0) : M<T>::div(num, den);
    return limiter<T>(lim, r) * den;
}

// Half slope .5 * phi(r) * dU of "plm cons" for a limiter fixed at compile
// time.  For the symmetric limiters (phi(r) = r phi(1/r)) the reference's
// selector between r = dUL/dUR and r = dUR/dUL (plm.cl:62-71) picks the same
// value either way, and phi(r) dU has a closed form in dUL and dUR that needs
// neither r nor the selector; all are zero unless dUL dUR > 0:
//   minmod             the one of dUL, dUR smaller in magnitude
//   monotized central  sign * min(2|dUL|, |dUL + dUR| / 2, 2|dUR|)
//   superbee           sign * max(min(|dUR|, 2|dUL|), min(2|dUR|, |dUL|))
//   van Leer (abs)     2 dUL dUR / (dUL + dUR)
// The table's van Leer keeps the general path: its 0/0 at r = -1 is behaviour
// the reference has.
template <typename T, int LIMC>
__device__ __forceinline__ T plmHalfSlopeD(T dUL, T dUR, int limRT) {
    if constexpr (LIMC == 8 || LIMC == 17 || LIMC == 18 || LIMC == 20) {
        T const prod = dUL * dUR;
        T h;
        if constexpr (LIMC == 8) {
            h = T(.5) * (M<T>::abs_(dUL) < M<T>::abs_(dUR) ? dUL : dUR);
        } else if constexpr (LIMC == 17) {
            T const a = M<T>::abs_(dUL), b = M<T>::abs_(dUR);
            T const m = tmin(tmin(a, b), T(.25) * M<T>::abs_(dUL + dUR));
            h = dUR < T(0) ? -m : m;
        } else if constexpr (LIMC == 18) {
            T const a = M<T>::abs_(dUL), b = M<T>::abs_(dUR);
            T const m = tmax(tmin(b, T(2) * a), tmin(T(2) * b, a));
            h = T(.5) * (dUR < T(0) ? -m : m);
        } else {
            h = M<T>::div(prod, dUL + dUR);
        }
        return prod > T(0) ? h : T(0);
    } else {
        return T(.5) * plmSigmaD<T>(dUL, dUR, LIMC >= 0 ? LIMC : limRT);
    }
}

}  // namespace fast
}  // namespace hc
