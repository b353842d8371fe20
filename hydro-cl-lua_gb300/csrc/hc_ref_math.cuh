// hc_ref_math.cuh -- the reference's per-interface and per-cell arithmetic in
// double precision, written term by term in the order hydro-cl-lua's
// generated OpenCL evaluates it (Euler equations, Cartesian chart with
// side-permutation normals).  Translation units that include this header are
// compiled with -fmad=false, so every product and sum is rounded separately.
//
//   limiter table          hydro/app.lua:614-635
//   calc_P, calc_Cs, ...   hydro/eqn/euler.cl:63-173
//   eigen_forInterface     hydro/eqn/euler.cl:347-430
//   eigen_left/rightTrans. hydro/eqn/euler.cl:434-542
//   Roe flux               hydro/flux/roe.cl:17-163
//   plm cons / prim / athena  hydro/solver/plm.cl:27-91, 191-253, 782-879
//   normals                hydro/coord/coord.lua:2341-2409
//   real3_dot              hydro/code/math.cl:172-181, 221
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace hc {
namespace ref {

struct Eos {
    double gamma, rhoMin, PMin;
    int fluxLimiter, slopeLimiter;
    int flux;   // HC_FLUX_*
    int hllcMethod;   // euler-hllc's hllcMethod, 0..2
    int recon;  // HC_RECON_*
    int entropyFix;        // Roe: useEntropyFluxFix
    double entropyFactor;  // its entropyFluxFixLimitingFactor
};

// OpenCL C max/min on floating types.
__host__ __device__ __forceinline__ double clmax(double x, double y) { return x < y ? y : x; }
__host__ __device__ __forceinline__ double clmin(double x, double y) { return y < x ? y : x; }

__device__ __forceinline__ double limiter(int which, double r) {
    switch (which) {
    case 0: return 0.;                                                              // donor cell
    case 1: return 1.;                                                              // Lax-Wendroff
    case 2: return r;                                                               // Beam-Warming
    case 3: return .5 * (1. + r);                                                   // Fromm
    case 4: return clmax(0., r) * (3. * r + 1.) / ((r + 1.) * (r + 1.));            // CHARM
    case 5: return clmax(0., 1.5 * (r + fabs(r)) / (r + 2.));                       // HCUS
    case 6: return clmax(0., 2. * (r + fabs(r)) / (r + 3.));                        // HQUICK
    case 7: return clmax(0., clmin(2. * r, clmin((1. + 2. * r) / 3., 2.)));         // Koren
    case 8: return clmax(0., clmin(r, 1.));                                         // minmod
    case 9: return clmax(0., clmin(r, 1.5));                                        // Oshker
    case 10: return .5 * (r * r + r) / (r * r + r + 1.);                            // ospre
    case 11: return clmax(0., clmin(2. * r, clmin(.25 + .75 * r, 4.)));             // smart
    case 12: return clmax(0., clmax(clmin(1.5 * r, 1.), clmin(r, 1.5)));            // Sweby
    case 13: return clmax(0., clmin(clmin(2. * r, .75 + .25 * r), clmin(.25 + .75 * r, 2.))); // UMIST
    case 14: return (r * r + r) / (r * r + 1.);                                     // van Albada 1
    case 15: return 2. * r / (r * r + 1.);                                          // van Albada 2
    case 16: return clmax(0., r) * 2. / (1. + r);                                   // van Leer
    case 17: return clmax(0., clmin(2., clmin(.5 * (1. + r), 2. * r)));             // monotized central
    case 18: return clmax(0., clmax(clmin(1., 2. * r), clmin(2., r)));             // superbee
    case 19: return .5 * (r + 1.) * clmin(1., clmin(4. * r / (r + 1.), 4. / (r + 1.))); // Barth-Jespersen
    case 20: return (r + fabs(r)) / (1. + fabs(r));                                 // van Leer, app.lua:631 comment
    }
    return 0.;
}

struct Eig { double rho, v[3], hTotal, Cs, vSq, vL[3]; };
struct Prim { double rho, v[3], P; };

// coordLenSq on the Cartesian chart: x*x + y*y + z*z, left to right.
__device__ __forceinline__ double lenSq(const double* v) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }
// real3_dot: x*x' + (y*y' + z*z').
__device__ __forceinline__ double dot3(const double* a, const double* b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }

__device__ __forceinline__ double calcP(const Eos& s, const double* U) {
    double const EKin = U[0] < s.rhoMin ? 0. : (.5 * lenSq(U + 1) / U[0]);
    return U[0] < s.rhoMin ? 0. : ((s.gamma - 1.) * (U[4] - EKin));
}

// primFromCons: the rhoMin-guarded branch is dead code in the reference; the
// unconditional assignments after it define the result.
__device__ __forceinline__ void primFromCons(Prim& W, const Eos& s, const double* U) {
    double const inv = 1. / U[0];
    W.rho = U[0];
    W.v[0] = U[1] * inv;
    W.v[1] = U[2] * inv;
    W.v[2] = U[3] * inv;
    W.P = calcP(s, U);
}

__device__ __forceinline__ double calcCs(const Eos& s, const Prim& W) {
    if (W.P <= s.PMin) return 0.;
    if (W.rho < s.rhoMin) return INFINITY;
    return sqrt(s.gamma * W.P / W.rho);
}

__device__ __forceinline__ void eigenForInterface(Eig& e, const Eos& s, const double* UL, const double* UR) {
    double const eps = 1e-5;
    bool const lv = UL[0] < eps, rv = UR[0] < eps;
    if (lv && rv) {
        e.rho = 0.; e.v[0] = e.v[1] = e.v[2] = 0.; e.vSq = 0.;
        e.vL[0] = e.vL[1] = e.vL[2] = 0.; e.hTotal = 0.; e.Cs = 0.;
        return;
    }
    if (lv || rv) {
        const double* Uo = lv ? UR : UL;
        Prim W;
        primFromCons(W, s, Uo);
        e.rho = Uo[0];
        for (int k = 0; k < 3; ++k) { e.v[k] = W.v[k]; e.vL[k] = W.v[k]; }
        e.vSq = dot3(W.v, e.vL);
        e.hTotal = (W.P + Uo[4]) / W.rho;
        e.Cs = calcCs(s, W);
        return;
    }
    Prim WL, WR;
    primFromCons(WL, s, UL);
    double const sqrtRhoL = sqrt(WL.rho);
    double const hTotalL = (WL.P + UL[4]) / WL.rho;
    primFromCons(WR, s, UR);
    double const sqrtRhoR = sqrt(WR.rho);
    double const hTotalR = (WR.P + UR[4]) / WR.rho;
    double const invDenom = 1. / (sqrtRhoL + sqrtRhoR);
    e.rho = sqrtRhoL * sqrtRhoR;
    double v[3];
    for (int k = 0; k < 3; ++k) v[k] = WL.v[k] * (sqrtRhoL * invDenom) + WR.v[k] * (sqrtRhoR * invDenom);
    double const hTotal = invDenom * (sqrtRhoL * hTotalL + sqrtRhoR * hTotalR);
    double const vSq = dot3(v, v);
    double const eKin = .5 * vSq;
    double const h = hTotal - eKin;
    if (h < eps) {
        e.hTotal = eKin;
        e.Cs = 0.;
    } else {
        e.hTotal = hTotal;
        e.Cs = sqrt((s.gamma - 1.) * h);
    }
    for (int k = 0; k < 3; ++k) { e.v[k] = v[k]; e.vL[k] = v[k]; }
    e.vSq = vSq;
}

// (n_j)_i = 1 when side == (i - j) mod 3 (1-based i, j), else 0.
__device__ __forceinline__ double nrm(int side, int j, int i) { return side == ((i - j + 3) % 3) ? 1. : 0.; }

__device__ __forceinline__ void leftTransform(double* w, const Eos& s, const Eig& e, const double* X, int side) {
    if (e.rho < s.rhoMin) {
        for (int j = 0; j < 5; ++j) w[j] = X[j];
        return;
    }
    double const vn0 = e.v[side], vn1 = e.v[(side + 1) % 3], vn2 = e.v[(side + 2) % 3];
    double const nLen = 1.;
    double const inv_nLen = 1. / nLen;
    double const denom = 2. * e.Cs * e.Cs;
    double const invDenom = 1. / denom;
    double const g1 = s.gamma - 1.;
    w[0] = (X[0] * (.5 * g1 * e.vSq + e.Cs * vn0 * inv_nLen)
          + X[1] * (-g1 * e.vL[0] - e.Cs * nrm(side, 1, 1))
          + X[2] * (-g1 * e.vL[1] - e.Cs * nrm(side, 1, 2))
          + X[3] * (-g1 * e.vL[2] - e.Cs * nrm(side, 1, 3))
          + X[4] * g1) * invDenom;
    w[1] = (X[0] * (denom - g1 * e.vSq)
          + X[1] * 2. * g1 * e.vL[0]
          + X[2] * 2. * g1 * e.vL[1]
          + X[3] * 2. * g1 * e.vL[2]
          + X[4] * -2. * g1) * invDenom;
    w[2] = X[0] * -vn1 + X[1] * nrm(side, 2, 1) + X[2] * nrm(side, 2, 2) + X[3] * nrm(side, 2, 3);
    w[3] = X[0] * -vn2 + X[1] * nrm(side, 3, 1) + X[2] * nrm(side, 3, 2) + X[3] * nrm(side, 3, 3);
    w[4] = (X[0] * (.5 * g1 * e.vSq - e.Cs * vn0 * inv_nLen)
          + X[1] * (-g1 * e.vL[0] + e.Cs * nrm(side, 1, 1))
          + X[2] * (-g1 * e.vL[1] + e.Cs * nrm(side, 1, 2))
          + X[3] * (-g1 * e.vL[2] + e.Cs * nrm(side, 1, 3))
          + X[4] * g1) * invDenom;
}

__device__ __forceinline__ void rightTransform(double* r, const Eos& s, const Eig& e, const double* X, int side) {
    if (e.rho < s.rhoMin) {
        for (int j = 0; j < 5; ++j) r[j] = X[j];
    } else {
        double const vn0 = e.v[side], vn1 = e.v[(side + 1) % 3], vn2 = e.v[(side + 2) % 3];
        double const nLen = 1.;
        double const inv_nLen = 1. / nLen;
        r[0] = X[0] + X[1] + X[4];
        for (int k = 0; k < 3; ++k) {
            int const i = k + 1;
            r[1 + k] = X[0] * (e.v[k] - e.Cs * nrm(side, 1, i))
                     + X[1] * e.v[k]
                     + X[2] * nrm(side, 2, i)
                     + X[3] * nrm(side, 3, i)
                     + X[4] * (e.v[k] + e.Cs * nrm(side, 1, i));
        }
        r[4] = X[0] * (e.hTotal - e.Cs * vn0 * inv_nLen)
             + X[1] * .5 * e.vSq
             + X[2] * vn1
             + X[3] * vn2
             + X[4] * (e.hTotal + e.Cs * vn0 * inv_nLen);
    }
    r[5] = 0.;
}

// Per-interface data the flux limiter reuses from the neighbouring
// interfaces: the Roe eigen-state and the projected jump L.(UR - UL).
struct Iface {
    Eig eig;
    double dW[5];
};

__device__ __forceinline__ void makeIface(Iface& I, const Eos& s, const double* UL, const double* UR, int side) {
    eigenForInterface(I.eig, s, UL, UR);
    double dU[6];
    for (int j = 0; j < 6; ++j) dU[j] = UR[j] - UL[j];
    leftTransform(I.dW, s, I.eig, dU, side);
}

// fluxFromCons (euler.cl:271-291): F = (rho v_n, m v_n + n P, (ETotal + P) v_n, 0)
// with n = normal_u1 = e_side for the Cartesian side normals (coord.lua:2378-2386).
__device__ __forceinline__ void fluxFromCons(double* F, const Eos& s, const double* U, int side) {
    Prim W;
    primFromCons(W, s, U);
    double const v_n = W.v[side];
    F[0] = U[0] * v_n;
    for (int i = 0; i < 3; ++i) F[1 + i] = U[1 + i] * v_n + (side == i ? 1. : 0.) * W.P;
    double const HTotal = U[4] + W.P;
    F[4] = HTotal * v_n;
    F[5] = 0.;
}

// Roe flux at the interface C between UL and UR (hydro/flux/roe.cl:17-163 with
// roeUseFluxFromCons, which Euler inherits from Equation, eqn.lua:46):
//   F = R.fluxEig + (F(UL) + F(UR)) / 2,
//   fluxEig_j = 0 - lambda_j dW_j (sgn lambda_j [+ phi (lambda_j dt/dx - sgn)]) / 2.
// With the flux limiter on, IL and IR are the interfaces one cell to the left
// and right (their eigen-states and projected jumps are the deltaUEigL /
// deltaUEigR the reference recomputes from the same inputs).
__device__ __forceinline__ void roeFlux(double* F, const Eos& s, const double* UL, const double* UR,
                                        const Iface& C, const Iface* IL, const Iface* IR,
                                        int side, bool lim, double dt_dx) {
    double const Cs_nLen = 1. * C.eig.Cs;
    double const v_n = C.eig.v[side];
    double fluxEig[5];
    for (int j = 0; j < 5; ++j) {
        double lambda = j == 0 ? v_n - Cs_nLen : (j == 4 ? v_n + Cs_nLen : v_n);
        if (s.entropyFix) {
            // useEntropyFluxFix (roe.cl:83-101): Harten's fix of the wave
            // speeds slower than factor * Cs; OpenCL's sign() keeps +-0
            double const dws = s.entropyFactor * C.eig.Cs;
            if (fabs(lambda) < dws) {
                double const sg = lambda > 0 ? 1. : (lambda < 0 ? -1. : lambda);
                lambda = sg * .5 * (lambda * lambda / dws + dws);
            }
        }
        fluxEig[j] = 0.;
        double const sgn = lambda >= 0 ? 1. : -1.;
        if (lim) {
            double rEig;
            if (C.dW[j] == 0) rEig = 0;
            else if (lambda >= 0) rEig = IL->dW[j] / C.dW[j];
            else rEig = IR->dW[j] / C.dW[j];
            double const phi = limiter(s.fluxLimiter, rEig);
            fluxEig[j] -= .5 * lambda * C.dW[j] * (sgn + phi * (lambda * dt_dx - sgn));
        } else {
            fluxEig[j] -= .5 * lambda * C.dW[j] * (sgn);
        }
    }
    rightTransform(F, s, C.eig, fluxEig, side);
    double FL[6], FR[6];
    fluxFromCons(FL, s, UL, side);
    fluxFromCons(FR, s, UR, side);
    for (int j = 0; j < 5; ++j) F[j] += .5 * (FL[j] + FR[j]);
}

// calc_Cs_fromCons (euler.cl:98-112)
__device__ __forceinline__ double calcCsFromCons(const Eos& s, const double* U) {
    double const P = calcP(s, U);
    if (P <= s.PMin) return 0.;
    if (U[0] < s.rhoMin) return INFINITY;
    return sqrt(s.gamma * P / U[0]);
}

// consWaveCodePrefix (euler.lua:329-337) with normal_len = 1: v_n -/+ Cs of one state
__device__ __forceinline__ void consWaveMinMax(const Eos& s, const double* U, int side, double& lmin, double& lmax) {
    double Cs_nLen = calcCsFromCons(s, U);
    Cs_nLen *= 1.;
    double const v_n = U[0] < s.rhoMin ? 0. : U[1 + side] / U[0];
    lmin = v_n - Cs_nLen;
    lmax = v_n + Cs_nLen;
}

// hydro/flux/rusanov.cl.  The bound lambdaMax is assigned per side in a loop
// over L then R, so the right state's value is the one used.
__device__ __forceinline__ void rusanovFlux(double* F, const Eos& s, const double* UL, const double* UR, int side) {
    double lmin, lmax;
    consWaveMinMax(s, UL, side, lmin, lmax);
    double lambdaMax = clmax(fabs(lmin), fabs(lmax));
    consWaveMinMax(s, UR, side, lmin, lmax);
    lambdaMax = clmax(fabs(lmin), fabs(lmax));
    double FL[6], FR[6];
    fluxFromCons(FL, s, UL, side);
    fluxFromCons(FR, s, UR, side);
    for (int j = 0; j < 5; ++j) F[j] = .5 * (FL[j] + FR[j] - lambdaMax * (UR[j] - UL[j]));
    F[5] = 0.;
}

// hydro/flux/hll.cl, hllCalcWaveMethod 'Davis direct bounded' (hll.lua:9).
// Returns false when sL or sR is NaN: no branch assigns the flux then.
__device__ __forceinline__ bool hllFlux(double* F, const Eos& s, const double* UL, const double* UR, int side,
                                        const Eig& eig) {
    double const Cs_nLen = 1. * eig.Cs;
    double const v_n = eig.v[side];
    double const lambdaIntMin = v_n - Cs_nLen;
    double const lambdaIntMax = v_n + Cs_nLen;
    double lambdaLMin, lambdaRMax, unused;
    consWaveMinMax(s, UL, side, lambdaLMin, unused);
    consWaveMinMax(s, UR, side, unused, lambdaRMax);
    double const sL = clmin(lambdaLMin, lambdaIntMin);
    double const sR = clmax(lambdaRMax, lambdaIntMax);
    if (0 <= sL) {
        fluxFromCons(F, s, UL, side);
    } else if (sR <= 0) {
        fluxFromCons(F, s, UR, side);
    } else if (sL <= 0 && 0 <= sR) {
        double FL[6], FR[6];
        fluxFromCons(FL, s, UL, side);
        fluxFromCons(FR, s, UR, side);
        for (int j = 0; j < 5; ++j) F[j] = (sR * FL[j] - sL * FR[j] + sL * sR * (UR[j] - UL[j])) / (sR - sL);
        F[5] = 0.;
    } else {
        return false;
    }
    return true;
}

// hydro/flux/euler-hllc.cl (2012 Toro's HLLC; hllcMethod 0, 1, 2; waves as
// hll.cl's 'Davis direct bounded').  Interface-frame vectors are
// normal_vecDotNs (v[side], v[side+1], v[side+2]), mapped back with
// normal_vecFromNs.  Returns false when no branch assigns the flux (NaN).
__device__ __forceinline__ void vecFromNs(double* out, int side, const double* v) {
    for (int i = 0; i < 3; ++i) out[i] = v[(3 - side + i) % 3];
}

__device__ __forceinline__ bool hllcFlux(double* flux, const Eos& s, const double* UL, const double* UR, int side,
                                         const Eig& eig) {
    Prim WL, WR;
    primFromCons(WL, s, UL);
    primFromCons(WR, s, UR);
    double const Cs_nLen = 1. * eig.Cs;
    double const v_n = eig.v[side];
    double const lambdaIntMin = v_n - Cs_nLen;
    double const lambdaIntMax = v_n + Cs_nLen;
    double lambdaLMin, lambdaRMax, unused;
    consWaveMinMax(s, UL, side, lambdaLMin, unused);
    consWaveMinMax(s, UR, side, unused, lambdaRMax);
    double const sL = clmin(lambdaLMin, lambdaIntMin);
    double const sR = clmax(lambdaRMax, lambdaIntMax);
    double const vnL[3] = {WL.v[side], WL.v[(side + 1) % 3], WL.v[(side + 2) % 3]};
    double const vnR[3] = {WR.v[side], WR.v[(side + 1) % 3], WR.v[(side + 2) % 3]};
    double const sStar = (WR.rho * vnR[0] * (sR - vnR[0]) - WL.rho * vnL[0] * (sL - vnL[0]) + WL.P - WR.P)
        / (WR.rho * (sR - vnR[0]) - WL.rho * (sL - vnL[0]));
    int const m = s.hllcMethod;
    // the star-region flux of one side (isL: the left one)
    auto star = [&](const double* U, const Prim& W, const double* vn, double sK, bool isL) {
        double F[6];
        fluxFromCons(F, s, U, side);
        if (m == 0) {
            double UStar[6];
            UStar[0] = U[0] * (sK - vn[0]) / (sK - sStar);
            double const vs[3] = {sStar, vn[1], vn[2]};
            double vStar[3];
            vecFromNs(vStar, side, vs);
            for (int i = 0; i < 3; ++i) UStar[1 + i] = UStar[0] * vStar[i];
            UStar[4] = UStar[0] * (U[4] / U[0] + (sStar - vn[0]) * (sStar + W.P / (U[0] * (sK - vn[0]))));
            UStar[5] = U[5];
            for (int i = 0; i < 6; ++i) flux[i] = F[i] + sK * (UStar[i] - U[i]);
            return;
        }
        double const Umn[3] = {U[1 + side], U[1 + (side + 1) % 3], U[1 + (side + 2) % 3]};
        double const Fmn[3] = {F[1 + side], F[1 + (side + 1) % 3], F[1 + (side + 2) % 3]};
        double mflux[3], out[3];
        if (m == 1) {
            flux[0] = (sStar * (sK * U[0] - F[0])) / (sK - sStar);
            mflux[0] = (sStar * (sK * Umn[0] - Fmn[0]) + sK * (W.P + W.rho * (sK - vn[0]) * (sStar - vn[0]))) / (sK - sStar);
            mflux[1] = (sStar * (sK * Umn[1] - Fmn[1])) / (sK - sStar);
            mflux[2] = (sStar * (sK * Umn[2] - Fmn[2])) / (sK - sStar);
            vecFromNs(out, side, mflux);
            for (int i = 0; i < 3; ++i) flux[1 + i] = out[i];
            flux[4] = (sStar * (sK * U[4] - F[4]) + sK * (W.P + W.rho * (sK - vn[0]) * (sStar - vn[0])) * sStar) / (sK - sStar);
        } else {
            double const PLR = .5 * (WL.P + WR.P + WL.rho * (sL - vnL[0]) * (sStar - vnL[0])
                                     + WR.rho * (sR - vnR[0]) * (sStar - vnR[0]));
            if (isL) {
                flux[0] = (sK * U[0] - F[0]) * sStar / (sK - sStar);
                mflux[0] = ((sK * Umn[0] - Fmn[0]) * sStar + sK * PLR) / (sK - sStar);
            } else {
                flux[0] = sStar * (sK * U[0] - F[0]) / (sK - sStar);
                mflux[0] = (sStar * (sK * Umn[0] - Fmn[0]) + sK * PLR) / (sK - sStar);
            }
            mflux[1] = sStar * (sK * Umn[1] - Fmn[1]) / (sK - sStar);
            mflux[2] = sStar * (sK * Umn[2] - Fmn[2]) / (sK - sStar);
            vecFromNs(out, side, mflux);
            for (int i = 0; i < 3; ++i) flux[1 + i] = out[i];
            flux[4] = (sStar * (sK * U[4] - F[4]) + sK * PLR * sStar) / (sK - sStar);
        }
    };
    if (0 <= sL) {
        fluxFromCons(flux, s, UL, side);
    } else if (sL <= 0. && 0. <= sStar) {
        star(UL, WL, vnL, sL, true);
    } else if (sStar <= 0. && 0. <= sR) {
        star(UR, WR, vnR, sR, false);
    } else if (sR <= 0) {
        fluxFromCons(flux, s, UR, side);
    } else if (sL <= 0 && 0 <= sR) {
        double FL[6], FR[6];
        fluxFromCons(FL, s, UL, side);
        fluxFromCons(FR, s, UR, side);
        for (int j = 0; j < 5; ++j) flux[j] = (sR * FL[j] - sL * FR[j] + sL * sR * (UR[j] - UL[j])) / (sR - sL);
        flux[5] = 0.;
    } else {
        return false;
    }
    return true;
}

// "plm cons" (hydro/solver/plm.cl:27-91): L and R states of the middle cell.
__device__ __forceinline__ void plmCons(double* L, double* R, const Eos& s, const double* Um, const double* U0, const double* Up) {
    for (int j = 0; j < 6; ++j) { L[j] = U0[j]; R[j] = U0[j]; }
    for (int j = 0; j < 5; ++j) {
        double const dUR = Up[j] - U0[j];
        double const dUL = U0[j] - Um[j];
        double sigma;
        double const dUC = .5 * (dUR - dUL);
        if (dUC >= 0) {
            double const r = dUR == 0 ? 0 : (dUL / dUR);
            sigma = limiter(s.slopeLimiter, r) * dUR;
        } else {
            double const r = dUL == 0 ? 0 : (dUR / dUL);
            sigma = limiter(s.slopeLimiter, r) * dUL;
        }
        R[j] += .5 * sigma;
        L[j] -= .5 * sigma;
    }
}

// OpenCL C sign(): 1 for x > 0, -1 for x < 0, x itself for +-0, 0 for NaN.
__device__ __forceinline__ double clsign(double x) { return x > 0 ? 1. : (x < 0 ? -1. : (x == 0 ? x : 0.)); }

// primFromCons as an array (rho, v.x, v.y, v.z, P) and consFromPrim back
// (euler.cl:140-173); ePot is carried separately.
__device__ __forceinline__ void primArr(double* w, const Eos& s, const double* U) {
    Prim W;
    primFromCons(W, s, U);
    w[0] = W.rho;
    w[1] = W.v[0];
    w[2] = W.v[1];
    w[3] = W.v[2];
    w[4] = W.P;
}
__device__ __forceinline__ void consArr(double* U, const Eos& s, const double* w, double ePot) {
    U[0] = w[0];
    U[1] = w[1] * w[0];
    U[2] = w[2] * w[0];
    U[3] = w[3] * w[0];
    U[4] = w[0] * (.5 * lenSq(w + 1)) + w[4] / (s.gamma - 1.);
    U[5] = ePot;
}

// "plm prim" (hydro/solver/plm.cl:191-253): the primitives' slopes,
// r = dWL / dWR, sigma = phi(r) dWR.
__device__ __forceinline__ void plmPrim(double* L, double* R, const Eos& s, const double* Um, const double* U0, const double* Up) {
    double W[5], WL[5], WR[5], nL[5], nR[5];
    primArr(W, s, U0);
    primArr(WL, s, Um);
    primArr(WR, s, Up);
    for (int j = 0; j < 5; ++j) {
        double const dWR = WR[j] - W[j];
        double const dWL = W[j] - WL[j];
        double const r = dWR == 0 ? 0 : (dWL / dWR);
        double const sigma = limiter(s.slopeLimiter, r) * dWR;
        nL[j] = W[j] - .5 * sigma;
        nR[j] = W[j] + .5 * sigma;
    }
    consArr(L, s, nL, U0[5]);
    consArr(R, s, nR, U0[5]);
}

// eigen_forCell (hydro/eqn/euler.cl:315-342)
__device__ __forceinline__ void eigenForCell(Eig& e, const Eos& s, const double* U) {
    Prim W;
    primFromCons(W, s, U);
    double const vL[3] = {W.v[0], W.v[1], W.v[2]};
    double const vSq = dot3(W.v, vL);
    double const eKin = .5 * vSq;
    double const hTotal = (W.P + U[4]) / W.rho;
    double const CsSq = (s.gamma - 1.) * (hTotal - eKin);
    e.rho = W.rho;
    for (int k = 0; k < 3; ++k) { e.v[k] = W.v[k]; e.vL[k] = vL[k]; }
    e.vSq = vSq;
    e.hTotal = hTotal;
    e.Cs = sqrt(CsSq);
}

// "plm athena", the first branch of that name (hydro/solver/plm.cl:782-879;
// the second, :950-968, is never reached): primitive differences projected
// with the cell's eigenvectors, limited per wave, projected back, clamped to
// the neighbouring primitives; the cell's L state is built from the
// right-edge value and its R state from the left-edge value, as
// plm.cl:877-878 assigns them.
__device__ __forceinline__ void plmAthena(double* L, double* R, const Eos& s, const double* Um, const double* U0,
                                          const double* Up, int side) {
    Eig eig;
    eigenForCell(eig, s, U0);
    double W[5], WL[5], WR[5];
    primArr(W, s, U0);
    primArr(WL, s, Um);
    primArr(WR, s, Up);
    double dWL[6], dWR[6], dWC[6], dWG[6];
    for (int j = 0; j < 5; ++j) {
        dWL[j] = W[j] - WL[j];
        dWR[j] = WR[j] - W[j];
        dWC[j] = .5 * (WR[j] - WL[j]);
        dWG[j] = (dWL[j] * dWR[j]) <= 0. ? 0. : (2. * dWL[j] * dWR[j] / (dWL[j] + dWR[j]));
    }
    dWL[5] = dWR[5] = dWC[5] = dWG[5] = 0.;
    double dal[5], dar[5], dac[5], dag[5];
    leftTransform(dal, s, eig, dWL, side);
    leftTransform(dar, s, eig, dWR, side);
    leftTransform(dac, s, eig, dWC, side);
    leftTransform(dag, s, eig, dWG, side);
    double da[5];
    for (int j = 0; j < 5; ++j) {
        da[j] = 0;
        if (dal[j] * dar[j] > 0) {
            double const s1 = clmin(fabs(dal[j]), fabs(dar[j]));
            double const s2 = clmin(fabs(dac[j]), fabs(dag[j]));
            da[j] = clsign(dac[j]) * clmin(2. * s1, s2);
        }
    }
    double dWm[6];
    rightTransform(dWm, s, eig, da, side);
    double lvs[5], rvs[5];
    for (int j = 0; j < 5; ++j) {
        double lv = W[j] - .5 * dWm[j];
        double rv = W[j] + .5 * dWm[j];
        double const C = rv + lv;
        lv = clmax(clmin(W[j], WL[j]), lv);
        lv = clmin(clmax(W[j], WL[j]), lv);
        rv = C - lv;
        rv = clmax(clmin(W[j], WR[j]), rv);
        rv = clmin(clmax(W[j], WR[j]), rv);
        lv = C - rv;
        lvs[j] = lv;
        rvs[j] = rv;
    }
    consArr(L, s, rvs, U0[5]);
    consArr(R, s, lvs, U0[5]);
}

// The cell's L and R states for the reconstruction s.recon along `side`
// ("piecewise constant": the cell itself).
__device__ __forceinline__ void plmAny(double* L, double* R, const Eos& s, const double* Um, const double* U0,
                                       const double* Up, int side) {
    switch (s.recon) {
    case 2: plmCons(L, R, s, Um, U0, Up); break;       // HC_RECON_PLM_CONS
    case 3: plmPrim(L, R, s, Um, U0, Up); break;       // HC_RECON_PLM_PRIM
    case 4: plmAthena(L, R, s, Um, U0, Up, side); break;   // HC_RECON_PLM_ATHENA
    default:
        for (int j = 0; j < 6; ++j) { L[j] = U0[j]; R[j] = U0[j]; }
    }
}

// constrainU (hydro/eqn/euler.cl:697-717) of one cell, in place.
__device__ __forceinline__ void constrain(double* U, const Eos& s) {
    if (U[0] < s.rhoMin) U[0] = s.rhoMin;
    Prim W;
    primFromCons(W, s, U);
    if (W.P < s.PMin) W.P = s.PMin;
    U[0] = W.rho;
    U[1] = W.v[0] * W.rho;
    U[2] = W.v[1] * W.rho;
    U[3] = W.v[2] * W.rho;
    U[4] = W.rho * (.5 * lenSq(W.v)) + W.P / (s.gamma - 1.);
}

// calcDTCell (hydro/eqn/cl/calcDT.cl:38-73) for one interior cell.
__device__ __forceinline__ double dtCell(const double* U, const Eos& s, int dim, const double* grid_dx) {
    double dt = INFINITY;
    double const P = calcP(s, U);
    double Cs;
    if (P <= s.PMin) Cs = 0.;
    else if (U[0] < s.rhoMin) Cs = INFINITY;
    else Cs = sqrt(s.gamma * P / U[0]);
    for (int side = 0; side < dim; ++side) {
        double const dx = grid_dx[side];
        if (dx > 0) {
            double const Cs_nLen = Cs * 1.;
            double const v_n = U[0] < s.rhoMin ? 0. : U[1 + side] / U[0];
            double const lmin = v_n - Cs_nLen;
            double const lmax = v_n + Cs_nLen;
            double a = clmax(fabs(lmin), fabs(lmax));
            a = clmax(1e-9, a);
            dt = clmin(dt, dx / a);
        }
    }
    return dt;
}

}  // namespace ref
}  // namespace hc
