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

// Roe flux at the interface C between UL and UR.  With the flux limiter on,
// IL and IR are the interfaces one cell to the left and right (their
// eigen-states and projected jumps are the deltaUEigL / deltaUEigR the
// reference recomputes from the same inputs).
__device__ __forceinline__ void roeFlux(double* F, const Eos& s, const double* UL, const double* UR,
                                        const Iface& C, const Iface* IL, const Iface* IR,
                                        int side, bool lim, double dt_dx) {
    double const Cs_nLen = 1. * C.eig.Cs;
    double const v_n = C.eig.v[side];
    double UAvg[6];
    for (int j = 0; j < 5; ++j) UAvg[j] = .5 * (UL[j] + UR[j]);
    UAvg[5] = 0.;
    double fluxEig[5];
    leftTransform(fluxEig, s, C.eig, UAvg, side);
    for (int j = 0; j < 5; ++j) {
        double const lambda = j == 0 ? v_n - Cs_nLen : (j == 4 ? v_n + Cs_nLen : v_n);
        fluxEig[j] *= lambda;
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
