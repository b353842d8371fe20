// hydro_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement, in plain C++ and double precision, of the finite-volume
// Euler update that hydro-cl-lua generates from its Lua/OpenCL templates for
// this option set: Euler equations, Cartesian chart (holonomic vectors,
// side-permutation normals), numGhost = 2, Roe flux (entropy fix off, the
// fluxFromCons form Euler inherits) with an optional flux limiter, HLL and
// Rusanov fluxes, optional "plm cons" reconstruction with a slope
// limiter, the freeflow / periodic / mirror boundaries, the explicit
// integrators (forward Euler and the Runge-Kutta tables), calcDT and
// constrainU, and the App's update loop (exit test before stepping, so the
// last step overshoots).
//
// It keeps the reference's array-of-structs cons_t layout (6 reals: rho, m.x,
// m.y, m.z, ETotal, ePot), its x-fastest indexing, its kernel domains and its
// expression order, so that a GPU form compiled without FMA contraction can be
// compared with it bit for bit.  It is built with -ffp-contract=off.
//
// Only the tests, the smoke check and the benchmark's CPU-baseline leg use
// this file.  The product library never links it.
//
// The reference cannot be run in this environment (LuaJIT and an OpenCL CPU
// platform are absent), so this restatement is pinned by the known-answer
// density L1 errors that the reference's own accuracy harness records
// (tests/test-order/schemes.lua) and by the eigen-decomposition identities
// the reference checks (hydro/solver/fvsolver.lua:396-527).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <limits>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef double real;

// hydro/eqn/euler.lua:166-171 -- cons_t = {rho, m[3], ETotal, ePot}
struct cons_t { real ptr[6]; };
// hydro/eqn/euler.lua:156-164 -- prim_t = {rho, v[3], P, ePot}
struct prim_t { real rho; real v[3]; real P; real ePot; };
// hydro/eqn/euler.lua:298-307 -- eigen_t
struct eigen_t { real rho; real v[3]; real hTotal; real Cs; real vSq; real vL[3]; };

enum { BC_NONE = 0, BC_PERIODIC = 1, BC_MIRROR = 2, BC_FREEFLOW = 3, BC_LINEAR = 4, BC_QUADRATIC = 5, BC_FIXED = 6 };
enum { RECON_NONE = 0, RECON_PIECEWISE_CONSTANT = 1, RECON_PLM_CONS = 2, RECON_PLM_PRIM = 3, RECON_PLM_ATHENA = 4 };
enum { FLUX_ROE = 0, FLUX_HLL = 1, FLUX_RUSANOV = 2, FLUX_HLLC = 3 };

// OpenCL C max/min on floating types: "returns y if x < y, otherwise x" and
// "returns y if y < x, otherwise x".
static inline real cl_max(real x, real y) { return x < y ? y : x; }
static inline real cl_min(real x, real y) { return y < x ? y : x; }

// hydro/app.lua:614-635 -- limiter table, 0-based (reference index - 1).
static real limiter(int which, real r) {
	switch (which) {
	case 0: return 0.;                                                        // donor cell
	case 1: return 1.;                                                        // Lax-Wendroff
	case 2: return r;                                                         // Beam-Warming
	case 3: return .5 * (1. + r);                                             // Fromm
	case 4: return cl_max(0., r) * (3. * r + 1.) / ((r + 1.) * (r + 1.));     // CHARM
	case 5: return cl_max(0., 1.5 * (r + std::fabs(r)) / (r + 2.));           // HCUS
	case 6: return cl_max(0., 2. * (r + std::fabs(r)) / (r + 3.));            // HQUICK
	case 7: return cl_max(0., cl_min(2. * r, cl_min((1. + 2. * r) / 3., 2.))); // Koren
	case 8: return cl_max(0., cl_min(r, 1.));                                 // minmod
	case 9: return cl_max(0., cl_min(r, 1.5));                                // Oshker
	case 10: return .5 * (r * r + r) / (r * r + r + 1.);                      // ospre
	case 11: return cl_max(0., cl_min(2. * r, cl_min(.25 + .75 * r, 4.)));    // smart
	case 12: return cl_max(0., cl_max(cl_min(1.5 * r, 1.), cl_min(r, 1.5)));  // Sweby
	case 13: return cl_max(0., cl_min(cl_min(2. * r, .75 + .25 * r), cl_min(.25 + .75 * r, 2.))); // UMIST
	case 14: return (r * r + r) / (r * r + 1.);                               // van Albada 1
	case 15: return 2. * r / (r * r + 1.);                                    // van Albada 2
	case 16: return cl_max(0., r) * 2. / (1. + r);                            // van Leer
	case 17: return cl_max(0., cl_min(2., cl_min(.5 * (1. + r), 2. * r)));    // monotized central
	case 18: return cl_max(0., cl_max(cl_min(1., 2. * r), cl_min(2., r)));    // superbee
	case 19: return .5 * (r + 1.) * cl_min(1., cl_min(4. * r / (r + 1.), 4. / (r + 1.))); // Barth-Jespersen
	// Not in the table: the van Leer form kept as a comment at app.lua:631.
	case 20: return (r + std::fabs(r)) / (1. + std::fabs(r));
	}
	return 0.;
}

// Runge-Kutta tables, hydro/int/all.lua:10-155.  Index 0 is forward Euler
// (hydro/int/fe.lua), which has its own integrate().
struct RKTable { int order; real alpha[4][4]; real beta[4][4]; };
static const RKTable rkTables[] = {
	{0, {{0}}, {{0}}},                                                   // 0 forward Euler
	{2, {{1,0},{1,0}}, {{.5,0},{0,1}}},                                  // 1 Runge-Kutta 2
	{2, {{1,0},{1,0}}, {{1,0},{.5,.5}}},                                 // 2 Runge-Kutta 2 Heun
	{2, {{1,0},{1,0}}, {{2./3.,0},{1./4.,3./4.}}},                       // 3 Runge-Kutta 2 Ralston
	{3, {{1,0,0},{1,0,0},{1,0,0}}, {{.5,0,0},{-1,2,0},{1./6.,2./6.,1./6.}}}, // 4 Runge-Kutta 3
	{4, {{1,0,0,0},{1,0,0,0},{1,0,0,0},{1,0,0,0}},
	    {{.5,0,0,0},{0,.5,0,0},{0,0,1,0},{1./6.,2./6.,2./6.,1./6.}}},   // 5 Runge-Kutta 4
	{4, {{1,0,0,0},{1,0,0,0},{1,0,0,0},{1,0,0,0}},
	    {{1./3.,0,0,0},{-1./3.,0,0,0},{1,-1,1,0},{1./8.,3./8.,3./8.,1./8.}}}, // 6 RK4 3/8ths rule
	{2, {{1,0},{.5,.5}}, {{1,0},{0,.5}}},                                // 7 Runge-Kutta 2, TVD
	{2, {{1,0},{1,0}}, {{-20,0},{41./40.,-1./40.}}},                     // 8 Runge-Kutta 2, non-TVD
	{3, {{1,0,0},{3./4.,1./4.,0},{1./3.,0,2./3.}}, {{1,0,0},{0,1./4.,0},{0,0,2./3.}}}, // 9 RK3 TVD
	{4, {{1,0,0,0},{649./1600.,951./1600.,0,0},{53989./2500000.,4806213./20000000.,23619./32000.,0},{1./5.,6127./30000.,7873./30000.,1./3.}},
	    {{.5,0,0,0},{-10890423./25193600.,5000./7873,0,0},{-102261./5000000.,-5121./20000.,7873./10000.,0},{1./10.,1./6.,0,1./6.}}}, // 10 RK4 TVD
	{4, {{1,0,0,0},{1,0,0,0},{1,0,0,0},{-1./3.,1./3.,2./3.,1./3.}},
	    {{.5,0,0,0},{0,.5,0,0},{0,0,1,0},{0,0,0,1./6.}}},               // 11 RK4 non-TVD
};
static const int numIntegrators = (int)(sizeof(rkTables) / sizeof(rkTables[0]));

struct Solver {
	// configuration
	int dim;
	int n[3];          // interior size per axis (1 for unused axes)
	int gs[3];         // gridSize with ghosts
	int stepsize[3];
	long numCells;
	real mins[3], maxs[3], grid_dx[3];
	int bc[6];         // xmin xmax ymin ymax zmin zmax
	int fluxLimiter, recon, slopeLimiter, integrator;
	int fluxType;      // FLUX_*
	int hllcMethod;    // euler-hllc's hllcMethod: 0, 1, 2
	real gamma, rhoMin, PMin, cfl, fixedDT;
	bool entropyFix;   // Roe: useEntropyFluxFix
	real entropyFactor;   // entropyFluxFixLimitingFactor
	real fixedCons[6][5];  // BC_FIXED sides: the ghost cells' state
	static const int numGhost = 2;

	// state
	real t;
	std::vector<cons_t> U, ULR, flux, reduce;
	std::vector<cons_t> UBufs[4], derivs[4];
	std::vector<real> dtBuf;
};

// ---------------------------------------------------------------------------
// hydro/eqn/euler.cl -- equation of state and conversions
// ---------------------------------------------------------------------------

// coordLenSq for the Cartesian chart (symmath output; summation order unpinned)
static inline real coordLenSq(const real v[3]) { return v[0] * v[0] + v[1] * v[1] + v[2] * v[2]; }
// hydro/code/math.cl:172-181,221 -- real3_dot = x*x' + (y*y' + z*z')
static inline real real3_dot(const real a[3], const real b[3]) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }

// euler.cl:63-67
static inline real calc_EKin_fromCons(const Solver& s, const cons_t& U) {
	return U.ptr[0] < s.rhoMin ? 0. : (.5 * coordLenSq(U.ptr + 1) / U.ptr[0]);
}
// euler.cl:79-83
static inline real calc_P(const Solver& s, const cons_t& U) {
	return U.ptr[0] < s.rhoMin ? 0. : ((s.gamma - 1.) * (U.ptr[4] - calc_EKin_fromCons(s, U)));
}
// euler.cl:87-94
static inline real calc_Cs(const Solver& s, const prim_t& W) {
	if (W.P <= s.PMin) return 0.;
	if (W.rho < s.rhoMin) return INFINITY;
	return std::sqrt(s.gamma * W.P / W.rho);
}
// euler.cl:98-112
static inline real calc_Cs_fromCons(const Solver& s, const cons_t& U) {
	real const P = calc_P(s, U);
	if (P <= s.PMin) return 0.;
	if (U.ptr[0] < s.rhoMin) return INFINITY;
	return std::sqrt(s.gamma * P / U.ptr[0]);
}
// euler.cl:25-29 / 18-21
static inline real calc_hTotal(real rho, real P, real ETotal) { return (P + ETotal) / rho; }

// euler.cl:140-159 (the first, rhoMin-guarded branch is overwritten by the
// unconditional assignments that follow it)
static inline void primFromCons(prim_t& W, const Solver& s, const cons_t& U) {
	real const invRho = 1. / U.ptr[0];
	W.rho = U.ptr[0];
	W.v[0] = U.ptr[1] * invRho;
	W.v[1] = U.ptr[2] * invRho;
	W.v[2] = U.ptr[3] * invRho;
	W.P = calc_P(s, U);
	W.ePot = U.ptr[5];
}
// euler.cl:163-173, 34-51, 69-75
static inline void consFromPrim(cons_t& U, const Solver& s, const prim_t& W) {
	U.ptr[0] = W.rho;
	U.ptr[1] = W.v[0] * W.rho;
	U.ptr[2] = W.v[1] * W.rho;
	U.ptr[3] = W.v[2] * W.rho;
	U.ptr[4] = W.rho * (.5 * coordLenSq(W.v)) + W.P / (s.gamma - 1.);
	U.ptr[5] = W.ePot;
}

// euler.cl:347-430
static void eigen_forInterface(eigen_t& e, const Solver& s, const cons_t& UL, const cons_t& UR) {
	real const rhoEpsilon = 1e-5;
	if (UL.ptr[0] < rhoEpsilon && UR.ptr[0] < rhoEpsilon) {
		e.rho = 0.;
		e.v[0] = e.v[1] = e.v[2] = 0.;
		e.vSq = 0.;
		e.vL[0] = e.vL[1] = e.vL[2] = 0.;
		e.hTotal = 0;
		e.Cs = 0;
	} else if (UL.ptr[0] < rhoEpsilon || UR.ptr[0] < rhoEpsilon) {
		// one side is vacuum: take the other side's state
		const cons_t& Uo = UL.ptr[0] < rhoEpsilon ? UR : UL;
		prim_t W;
		primFromCons(W, s, Uo);
		e.rho = Uo.ptr[0];
		for (int k = 0; k < 3; ++k) { e.v[k] = W.v[k]; e.vL[k] = W.v[k]; }
		e.vSq = real3_dot(W.v, e.vL);
		e.hTotal = calc_hTotal(W.rho, W.P, Uo.ptr[4]);
		e.Cs = calc_Cs(s, W);
	} else {
		prim_t WL, WR;
		primFromCons(WL, s, UL);
		real const sqrtRhoL = std::sqrt(WL.rho);
		real const hTotalL = calc_hTotal(WL.rho, WL.P, UL.ptr[4]);
		primFromCons(WR, s, UR);
		real const sqrtRhoR = std::sqrt(WR.rho);
		real const hTotalR = calc_hTotal(WR.rho, WR.P, UR.ptr[4]);
		real const invDenom = 1. / (sqrtRhoL + sqrtRhoR);
		e.rho = sqrtRhoL * sqrtRhoR;
		real v[3];
		for (int k = 0; k < 3; ++k) v[k] = WL.v[k] * (sqrtRhoL * invDenom) + WR.v[k] * (sqrtRhoR * invDenom);
		real const hTotal = invDenom * (sqrtRhoL * hTotalL + sqrtRhoR * hTotalR);
		real const vSq = real3_dot(v, v);
		real const eKin = .5 * vSq;
		real const h = hTotal - eKin;
		if (h < rhoEpsilon) {
			e.hTotal = eKin;
			e.Cs = 0.;
		} else {
			e.hTotal = hTotal;
			real const CsSq = (s.gamma - 1.) * h;
			e.Cs = std::sqrt(CsSq);
		}
		for (int k = 0; k < 3; ++k) { e.v[k] = v[k]; e.vL[k] = v[k]; }
		e.vSq = vSq;
	}
}

// Cartesian side normals, hydro/coord/coord.lua:2341-2409:
// (n_j)_i = 1 if side == (i - j) mod 3 else 0 (i, j 1-based).
static inline real nrm(int side, int j, int i) { return side == (((i - j) % 3) + 3) % 3 ? 1. : 0.; }

// euler.cl:434-489
static void eigen_leftTransform(real result[5], const Solver& s, const eigen_t& e, const real X[6], int side) {
	if (e.rho < s.rhoMin) {
		for (int j = 0; j < 5; ++j) result[j] = X[j];
		return;
	}
	real const v_n[3] = { e.v[side], e.v[(side + 1) % 3], e.v[(side + 2) % 3] };
	real const nLen = 1.;
	real const inv_nLen = 1. / nLen;
	real const denom = 2. * e.Cs * e.Cs;
	real const invDenom = 1. / denom;
	real const gamma_1 = s.gamma - 1.;
	result[0] = (
		X[0] * (.5 * gamma_1 * e.vSq + e.Cs * v_n[0] * inv_nLen)
		+ X[1] * (-gamma_1 * e.vL[0] - e.Cs * nrm(side, 1, 1))
		+ X[2] * (-gamma_1 * e.vL[1] - e.Cs * nrm(side, 1, 2))
		+ X[3] * (-gamma_1 * e.vL[2] - e.Cs * nrm(side, 1, 3))
		+ X[4] * gamma_1
	) * invDenom;
	result[1] = (
		X[0] * (denom - gamma_1 * e.vSq)
		+ X[1] * 2. * gamma_1 * e.vL[0]
		+ X[2] * 2. * gamma_1 * e.vL[1]
		+ X[3] * 2. * gamma_1 * e.vL[2]
		+ X[4] * -2. * gamma_1
	) * invDenom;
	result[2] =
		X[0] * -v_n[1]
		+ X[1] * nrm(side, 2, 1)
		+ X[2] * nrm(side, 2, 2)
		+ X[3] * nrm(side, 2, 3);
	result[3] =
		X[0] * -v_n[2]
		+ X[1] * nrm(side, 3, 1)
		+ X[2] * nrm(side, 3, 2)
		+ X[3] * nrm(side, 3, 3);
	result[4] = (
		X[0] * (.5 * gamma_1 * e.vSq - e.Cs * v_n[0] * inv_nLen)
		+ X[1] * (-gamma_1 * e.vL[0] + e.Cs * nrm(side, 1, 1))
		+ X[2] * (-gamma_1 * e.vL[1] + e.Cs * nrm(side, 1, 2))
		+ X[3] * (-gamma_1 * e.vL[2] + e.Cs * nrm(side, 1, 3))
		+ X[4] * gamma_1
	) * invDenom;
}

// euler.cl:493-542
static void eigen_rightTransform(real result[6], const Solver& s, const eigen_t& e, const real X[5], int side) {
	if (e.rho < s.rhoMin) {
		for (int j = 0; j < 5; ++j) result[j] = X[j];
	} else {
		real const v_n[3] = { e.v[side], e.v[(side + 1) % 3], e.v[(side + 2) % 3] };
		real const nLen = 1.;
		real const inv_nLen = 1. / nLen;
		result[0] = X[0] + X[1] + X[4];
		for (int k = 0; k < 3; ++k) {
			int const i = k + 1;  // 1-based axis index
			result[1 + k] =
				X[0] * (e.v[k] - e.Cs * nrm(side, 1, i))
				+ X[1] * e.v[k]
				+ X[2] * nrm(side, 2, i)
				+ X[3] * nrm(side, 3, i)
				+ X[4] * (e.v[k] + e.Cs * nrm(side, 1, i));
		}
		result[4] =
			X[0] * (e.hTotal - e.Cs * v_n[0] * inv_nLen)
			+ X[1] * .5 * e.vSq
			+ X[2] * v_n[1]
			+ X[3] * v_n[2]
			+ X[4] * (e.hTotal + e.Cs * v_n[0] * inv_nLen);
	}
	result[5] = 0;
}

// euler.cl:271-291 (fluxFromCons): F = (rho v_n, m v_n + n P, (ETotal + P) v_n, 0)
// with n = normal_u1 = e_side for the Cartesian side normals (coord.lua:2378-2386)
static void fluxFromCons(cons_t& F, const Solver& s, const cons_t& U, int side) {
	prim_t W;
	primFromCons(W, s, U);
	real const v_n = W.v[side];
	F.ptr[0] = U.ptr[0] * v_n;
	for (int i = 0; i < 3; ++i) F.ptr[1 + i] = U.ptr[1 + i] * v_n + (side == i ? 1. : 0.) * W.P;
	real const HTotal = U.ptr[4] + W.P;
	F.ptr[4] = HTotal * v_n;
	F.ptr[5] = 0;
}

// OpenCL C sign(): 1 for x > 0, -1 for x < 0, x itself for +-0, 0 for NaN.
static inline real clSign(real x) { return x > 0 ? 1. : (x < 0 ? -1. : (x == 0 ? x : 0.)); }

// hydro/flux/roe.cl:17-163 with roeUseFluxFromCons: Euler does not set it and
// inherits Equation.roeUseFluxFromCons = true (hydro/eqn/eqn.lua:46), so the
// flux is R.fluxEig + (F(UL) + F(UR)) / 2 with
// fluxEig_j = 0 - lambda_j dW_j (sgn + phi (lambda_j dt/dx - sgn)) / 2.  With
// useEntropyFluxFix (roe.cl:83-101) each lambda_j with |lambda_j| < factor Cs
// is first replaced by sign(lambda_j) (lambda_j^2 / dws + dws) / 2, dws =
// factor Cs; sgn and the flux limiter's ratio then follow the new value.
static void roeFluxForInterface(
	cons_t& resultFlux, const Solver& s,
	const cons_t& UL, const cons_t& UR, int side, bool useFluxLimiter, real dt_dx,
	const cons_t* UL_L, const cons_t* UL_R, const cons_t* UR_L, const cons_t* UR_R
) {
	eigen_t eig;
	eigen_forInterface(eig, s, UL, UR);
	real const Cs_nLen = 1. * eig.Cs;
	real const v_n = eig.v[side];

	real fluxEig[5];

	real deltaU[6], deltaUL[6], deltaUR[6];
	for (int j = 0; j < 6; ++j) {
		deltaU[j] = UR.ptr[j] - UL.ptr[j];
		if (useFluxLimiter) {
			deltaUL[j] = UR_L->ptr[j] - UL_L->ptr[j];
			deltaUR[j] = UR_R->ptr[j] - UL_R->ptr[j];
		}
	}
	real deltaUEig[5], deltaUEigL[5], deltaUEigR[5];
	eigen_leftTransform(deltaUEig, s, eig, deltaU, side);
	if (useFluxLimiter) {
		eigen_t eigL, eigR;
		eigen_forInterface(eigL, s, *UL_L, *UR_L);
		eigen_forInterface(eigR, s, *UL_R, *UR_R);
		eigen_leftTransform(deltaUEigL, s, eigL, deltaUL, side);
		eigen_leftTransform(deltaUEigR, s, eigR, deltaUR, side);
	}

	real const speedOfSound = eig.Cs;
	for (int j = 0; j < 5; ++j) {
		real lambda = j == 0 ? v_n - Cs_nLen : (j == 4 ? v_n + Cs_nLen : v_n);
		if (s.entropyFix) {
			real const dws = s.entropyFactor * speedOfSound;
			if (fabs(lambda) < dws) lambda = clSign(lambda) * .5 * (lambda * lambda / dws + dws);
		}
		fluxEig[j] = 0.;
		real const sgnLambda = lambda >= 0 ? 1 : -1;
		if (useFluxLimiter) {
			real rEig;
			if (deltaUEig[j] == 0) {
				rEig = 0;
			} else if (lambda >= 0) {
				rEig = deltaUEigL[j] / deltaUEig[j];
			} else {
				rEig = deltaUEigR[j] / deltaUEig[j];
			}
			real const phi = limiter(s.fluxLimiter, rEig);
			fluxEig[j] -= .5 * lambda * deltaUEig[j] * (sgnLambda + phi * (lambda * dt_dx - sgnLambda));
		} else {
			fluxEig[j] -= .5 * lambda * deltaUEig[j] * (sgnLambda);
		}
	}
	eigen_rightTransform(resultFlux.ptr, s, eig, fluxEig, side);
	cons_t FL, FR;
	fluxFromCons(FL, s, UL, side);
	fluxFromCons(FR, s, UR, side);
	for (int j = 0; j < 5; ++j) resultFlux.ptr[j] += .5 * (FL.ptr[j] + FR.ptr[j]);
}

// euler.lua:329-337 (consWaveCodePrefix) with normal_len = 1: the slowest and
// fastest waves v_n -/+ Cs of one conserved state
static inline void consWaveMinMax(const Solver& s, const cons_t& U, int side, real& lmin, real& lmax) {
	real Cs_nLen = calc_Cs_fromCons(s, U);
	Cs_nLen *= 1.;
	real const v_n = U.ptr[0] < s.rhoMin ? 0. : U.ptr[1 + side] / U.ptr[0];
	lmin = v_n - Cs_nLen;
	lmax = v_n + Cs_nLen;
}

// OpenCL max / min on reals (x < y ? y : x, y < x ? y : x)
static inline real clMax(real x, real y) { return x < y ? y : x; }
static inline real clMin(real x, real y) { return y < x ? y : x; }

// hydro/flux/rusanov.cl: the wave bound lambdaMax is assigned once per side in
// a loop over L then R, so the right state's value is the one used.
static void rusanovFluxForInterface(cons_t& resultFlux, const Solver& s, const cons_t& UL, const cons_t& UR, int side) {
	real lambdaMax = 0;
	{
		real lmin, lmax;
		consWaveMinMax(s, UL, side, lmin, lmax);
		lambdaMax = clMax(std::fabs(lmin), std::fabs(lmax));
	}
	{
		real lmin, lmax;
		consWaveMinMax(s, UR, side, lmin, lmax);
		lambdaMax = clMax(std::fabs(lmin), std::fabs(lmax));
	}
	cons_t FL, FR;
	fluxFromCons(FL, s, UL, side);
	fluxFromCons(FR, s, UR, side);
	for (int j = 0; j < 5; ++j)
		resultFlux.ptr[j] = .5 * (FL.ptr[j] + FR.ptr[j] - lambdaMax * (UR.ptr[j] - UL.ptr[j]));
}

// hydro/flux/hll.cl with hllCalcWaveMethod = 'Davis direct bounded' (hll.lua:9):
// sL = min(v_n - Cs of UL, Roe-average v_n - Cs), sR = max(v_n + Cs of UR,
// Roe-average v_n + Cs).  When sL or sR is NaN no branch assigns the flux and
// the flux buffer keeps its previous content, as in the reference.
static void hllFluxForInterface(cons_t& resultFlux, const Solver& s, const cons_t& UL, const cons_t& UR, int side) {
	eigen_t eigInt;
	eigen_forInterface(eigInt, s, UL, UR);
	real const Cs_nLen = 1. * eigInt.Cs;
	real const v_n = eigInt.v[side];
	real const lambdaIntMin = v_n - Cs_nLen;
	real const lambdaIntMax = v_n + Cs_nLen;
	real lambdaLMin, lambdaRMax, unused;
	consWaveMinMax(s, UL, side, lambdaLMin, unused);
	consWaveMinMax(s, UR, side, unused, lambdaRMax);
	real const sL = clMin(lambdaLMin, lambdaIntMin);
	real const sR = clMax(lambdaRMax, lambdaIntMax);
	if (0 <= sL) {
		fluxFromCons(resultFlux, s, UL, side);
	} else if (sR <= 0) {
		fluxFromCons(resultFlux, s, UR, side);
	} else if (sL <= 0 && 0 <= sR) {
		cons_t FL, FR;
		fluxFromCons(FL, s, UL, side);
		fluxFromCons(FR, s, UR, side);
		for (int j = 0; j < 5; ++j)
			resultFlux.ptr[j] = (sR * FL.ptr[j] - sL * FR.ptr[j] + sL * sR * (UR.ptr[j] - UL.ptr[j])) / (sR - sL);
	}
}

// hydro/flux/euler-hllc.cl (2012 Toro's HLLC, hllcMethod 0 / 1 / 2; waves
// as hll.cl's 'Davis direct bounded').  Vectors in the interface frame:
// vn = normal_vecDotNs(n, v) = (v[side], v[side+1], v[side+2]); back to
// the global frame with normal_vecFromNs (coord.lua:2392-2407).
static inline void vecFromNs(real out[3], int side, const real v[3]) {
	for (int i = 0; i < 3; ++i) out[i] = v[(3 - side + i) % 3];
}
static void hllcFluxForInterface(cons_t& flux, const Solver& s, const cons_t& UL, const cons_t& UR, int side) {
	prim_t WL, WR;
	primFromCons(WL, s, UL);
	primFromCons(WR, s, UR);
	eigen_t eigInt;
	eigen_forInterface(eigInt, s, UL, UR);
	real const Cs_nLen = 1. * eigInt.Cs;
	real const v_n = eigInt.v[side];
	real const lambdaIntMin = v_n - Cs_nLen;
	real const lambdaIntMax = v_n + Cs_nLen;
	real lambdaLMin, lambdaRMax, unused;
	consWaveMinMax(s, UL, side, lambdaLMin, unused);
	consWaveMinMax(s, UR, side, unused, lambdaRMax);
	real const sL = clMin(lambdaLMin, lambdaIntMin);
	real const sR = clMax(lambdaRMax, lambdaIntMax);
	real const vnL[3] = {WL.v[side], WL.v[(side + 1) % 3], WL.v[(side + 2) % 3]};
	real const vnR[3] = {WR.v[side], WR.v[(side + 1) % 3], WR.v[(side + 2) % 3]};
	real const sStar = (WR.rho * vnR[0] * (sR - vnR[0]) - WL.rho * vnL[0] * (sL - vnL[0]) + WL.P - WR.P)
		/ (WR.rho * (sR - vnR[0]) - WL.rho * (sL - vnL[0]));
	int const m = s.hllcMethod;
	// one side of the star region: X = L (sgn 0) or R
	auto star = [&](const cons_t& U, const prim_t& W, const real* vn, real sK) {
		cons_t F;
		fluxFromCons(F, s, U, side);
		if (m == 0) {
			cons_t UStar;
			UStar.ptr[0] = U.ptr[0] * (sK - vn[0]) / (sK - sStar);
			real const vs[3] = {sStar, vn[1], vn[2]};
			real vStar[3];
			vecFromNs(vStar, side, vs);
			for (int i = 0; i < 3; ++i) UStar.ptr[1 + i] = UStar.ptr[0] * vStar[i];
			UStar.ptr[4] = UStar.ptr[0] * (U.ptr[4] / U.ptr[0] + (sStar - vn[0]) * (sStar + W.P / (U.ptr[0] * (sK - vn[0]))));
			UStar.ptr[5] = U.ptr[5];   // never set by the reference; its flux is not used
			for (int i = 0; i < 6; ++i) flux.ptr[i] = F.ptr[i] + sK * (UStar.ptr[i] - U.ptr[i]);
			return;
		}
		real const Umn[3] = {U.ptr[1 + side], U.ptr[1 + (side + 1) % 3], U.ptr[1 + (side + 2) % 3]};
		real const Fmn[3] = {F.ptr[1 + side], F.ptr[1 + (side + 1) % 3], F.ptr[1 + (side + 2) % 3]};
		real mflux[3], out[3];
		if (m == 1) {
			flux.ptr[0] = (sStar * (sK * U.ptr[0] - F.ptr[0])) / (sK - sStar);
			mflux[0] = (sStar * (sK * Umn[0] - Fmn[0]) + sK * (W.P + W.rho * (sK - vn[0]) * (sStar - vn[0]))) / (sK - sStar);
			mflux[1] = (sStar * (sK * Umn[1] - Fmn[1])) / (sK - sStar);
			mflux[2] = (sStar * (sK * Umn[2] - Fmn[2])) / (sK - sStar);
			vecFromNs(out, side, mflux);
			for (int i = 0; i < 3; ++i) flux.ptr[1 + i] = out[i];
			flux.ptr[4] = (sStar * (sK * U.ptr[4] - F.ptr[4]) + sK * (W.P + W.rho * (sK - vn[0]) * (sStar - vn[0])) * sStar) / (sK - sStar);
		} else {
			real const PLR = .5 * (WL.P + WR.P + WL.rho * (sL - vnL[0]) * (sStar - vnL[0]) + WR.rho * (sR - vnR[0]) * (sStar - vnR[0]));
			// the left branch writes (sL rho - F rho) sStar / (..), the right one sStar (sR rho - F rho) / (..)
			if (&U == &UL) flux.ptr[0] = (sK * U.ptr[0] - F.ptr[0]) * sStar / (sK - sStar);
			else flux.ptr[0] = sStar * (sK * U.ptr[0] - F.ptr[0]) / (sK - sStar);
			mflux[0] = ((sK * Umn[0] - Fmn[0]) * sStar + sK * PLR) / (sK - sStar);
			if (&U == &UL) {
				mflux[1] = sStar * (sK * Umn[1] - Fmn[1]) / (sK - sStar);
				mflux[2] = sStar * (sK * Umn[2] - Fmn[2]) / (sK - sStar);
			} else {
				mflux[0] = (sStar * (sK * Umn[0] - Fmn[0]) + sK * PLR) / (sK - sStar);
				mflux[1] = sStar * (sK * Umn[1] - Fmn[1]) / (sK - sStar);
				mflux[2] = sStar * (sK * Umn[2] - Fmn[2]) / (sK - sStar);
			}
			vecFromNs(out, side, mflux);
			for (int i = 0; i < 3; ++i) flux.ptr[1 + i] = out[i];
			flux.ptr[4] = (sStar * (sK * U.ptr[4] - F.ptr[4]) + sK * PLR * sStar) / (sK - sStar);
		}
	};
	if (0 <= sL) {
		fluxFromCons(flux, s, UL, side);
	} else if (sL <= 0. && 0. <= sStar) {
		star(UL, WL, vnL, sL);
	} else if (sStar <= 0. && 0. <= sR) {
		star(UR, WR, vnR, sR);
	} else if (sR <= 0) {
		fluxFromCons(flux, s, UR, side);
	} else if (sL <= 0 && 0 <= sR) {
		cons_t FL, FR;
		fluxFromCons(FL, s, UL, side);
		fluxFromCons(FR, s, UR, side);
		for (int j = 0; j < 5; ++j)
			flux.ptr[j] = (sR * FL.ptr[j] - sL * FR.ptr[j] + sL * sR * (UR.ptr[j] - UL.ptr[j])) / (sR - sL);
	}
}

// ---------------------------------------------------------------------------
// index domains, hydro/solver/gridsolver.lua:277-320
// ---------------------------------------------------------------------------

static inline bool OOB(const Solver& s, const int i[3], int lhs, int rhs) {
	for (int d = 0; d < s.dim; ++d)
		if (i[d] < lhs || i[d] >= s.gs[d] - rhs) return true;
	return false;
}
static inline long INDEX(const Solver& s, int x, int y, int z) {
	return (long)x + (long)s.gs[0] * ((long)y + (long)s.gs[1] * (long)z);
}

template<typename F>
static void forAllCells(const Solver& s, F f) {
	long const n = s.numCells;
#pragma omp parallel for schedule(static)
	for (long index = 0; index < n; ++index) {
		int i[3];
		i[0] = (int)(index % s.gs[0]);
		i[1] = (int)((index / s.gs[0]) % s.gs[1]);
		i[2] = (int)(index / ((long)s.gs[0] * s.gs[1]));
		f(i, index);
	}
}

// ---------------------------------------------------------------------------
// boundary, hydro/solver/gridsolver.lua:638-780, 1070-1213, 1272-1320
// ---------------------------------------------------------------------------

static void boundary(Solver& s) {
	int const G = Solver::numGhost;
	for (int side = 0; side < s.dim; ++side) {
		int const gsSide = s.gs[side];
		int const N = gsSide - 2 * G;
		int o1 = (side + 1) % 3, o2 = (side + 2) % 3;
		// the other axes are looped over their full extent, ghosts included
		int const n1 = s.gs[o1], n2 = s.gs[o2];
		for (int b = 0; b < n2; ++b) for (int a = 0; a < n1; ++a) {
			auto at = [&](int j) -> cons_t& {
				int c[3]; c[side] = j; c[o1] = a; c[o2] = b;
				return s.U[INDEX(s, c[0], c[1], c[2])];
			};
			for (int j = 0; j < G; ++j) {
				for (int mm = 0; mm < 2; ++mm) {
					int const method = s.bc[2 * side + mm];
					int dst = -1, src = -1;
					if (method == BC_PERIODIC) {
						if (mm == 0) { dst = j; src = G + (j - G + 2 * N) % N; }
						else { dst = gsSide - 1 - j; src = G + (G - 1 - j) % N; }
					} else if (method == BC_MIRROR) {
						if (mm == 0) { dst = j; src = 2 * G - 1 - j; }
						else { dst = gsSide - G + j; src = gsSide - G - 1 - j; }
					} else if (method == BC_FREEFLOW) {
						if (mm == 0) { dst = j; src = G; }
						else { dst = gsSide - G + j; src = gsSide - G - 1; }
					} else if (method == BC_FIXED) {
						// gridsolver.lua:746-765: the side's ghosts take the
						// constant state fixedCode writes (consFromPrim, ePot 0)
						cons_t& d = at(mm == 0 ? j : gsSide - G + j);
						for (int k = 0; k < 5; ++k) d.ptr[k] = s.fixedCons[2 * side + mm][k];
						d.ptr[5] = 0.;
						continue;
					} else if (method == BC_LINEAR || method == BC_QUADRATIC) {
						// gridsolver.lua:783-858: outward from the interior, each
						// ghost from the two (three) cells inside it, all 6 reals
						int d, i1, i2, i3;
						if (mm == 0) { d = G - j - 1; i1 = G - j; i2 = G - j + 1; i3 = G - j + 2; }
						else { d = gsSide - G + j; i1 = gsSide - G + j - 1; i2 = gsSide - G + j - 2; i3 = gsSide - G + j - 3; }
						for (int k = 0; k < 6; ++k) {
							if (method == BC_LINEAR) at(d).ptr[k] = 2. * at(i1).ptr[k] - at(i2).ptr[k];
							else at(d).ptr[k] = 3. * at(i1).ptr[k] - 3. * at(i2).ptr[k] + at(i3).ptr[k];
						}
						continue;
					} else {
						continue;
					}
					at(dst) = at(src);
					if (method == BC_MIRROR) {
						// reflectVars.mirror (hydro/eqn/eqn.lua:366-370), restitution 1
						cons_t& d = at(dst);
						d.ptr[1 + side] = -1. * d.ptr[1 + side];
					}
				}
			}
		}
	}
}

// hydro/eqn/euler.cl:697-717 + hydro/solver/solverbase.lua:2116-2128
static void constrainU(Solver& s) {
	forAllCells(s, [&](const int*, long index) {
		cons_t& U = s.U[index];
		if (U.ptr[0] < s.rhoMin) U.ptr[0] = s.rhoMin;
		prim_t W;
		primFromCons(W, s, U);
		if (W.P < s.PMin) W.P = s.PMin;
		consFromPrim(U, s, W);
	});
	boundary(s);
}

static inline real& primAt(prim_t& W, int j) { return j == 0 ? W.rho : (j < 4 ? W.v[j - 1] : (j == 4 ? W.P : W.ePot)); }

// "plm cons", hydro/solver/plm.cl:27-91
static void plmCons(cons_t& L, cons_t& R, const Solver& s, const cons_t& UL, const cons_t& U, const cons_t& UR) {
	L = U;
	R = U;
	for (int j = 0; j < 5; ++j) {
		real const dUR = UR.ptr[j] - U.ptr[j];
		real const dUL = U.ptr[j] - UL.ptr[j];
		real sigma;
		real const dUC = .5 * (dUR - dUL);
		if (dUC >= 0) {
			real const r = dUR == 0 ? 0 : (dUL / dUR);
			real const phi = limiter(s.slopeLimiter, r);
			sigma = phi * dUR;
		} else {
			real const r = dUL == 0 ? 0 : (dUR / dUL);
			real const phi = limiter(s.slopeLimiter, r);
			sigma = phi * dUL;
		}
		R.ptr[j] += .5 * sigma;
		L.ptr[j] -= .5 * sigma;
	}
}

// "plm prim", hydro/solver/plm.cl:191-253: slopes of the primitives,
// r = dWL / dWR, sigma = phi(r) dWR
static void plmPrim(cons_t& L, cons_t& R, const Solver& s, const cons_t& UL, const cons_t& U, const cons_t& UR) {
	prim_t W, WL, WR;
	primFromCons(W, s, U);
	primFromCons(WL, s, UL);
	primFromCons(WR, s, UR);
	prim_t nWL = W, nWR = W;
	for (int j = 0; j < 5; ++j) {
		real const dWR = primAt(WR, j) - primAt(W, j);
		real const dWL = primAt(W, j) - primAt(WL, j);
		real const r = dWR == 0 ? 0 : (dWL / dWR);
		real const phi = limiter(s.slopeLimiter, r);
		real const sigma = phi * dWR;
		primAt(nWL, j) -= .5 * sigma;
		primAt(nWR, j) += .5 * sigma;
	}
	consFromPrim(L, s, nWL);
	consFromPrim(R, s, nWR);
}

// eigen_forCell, hydro/eqn/euler.cl:315-342
static void eigen_forCell(eigen_t& e, const Solver& s, const cons_t& U) {
	prim_t W;
	primFromCons(W, s, U);
	real vL[3] = { W.v[0], W.v[1], W.v[2] };
	real const vSq = real3_dot(W.v, vL);
	real const eKin = .5 * vSq;
	real const hTotal = calc_hTotal(W.rho, W.P, U.ptr[4]);
	real const CsSq = (s.gamma - 1.) * (hTotal - eKin);
	real const Cs = std::sqrt(CsSq);
	e.rho = W.rho;
	for (int k = 0; k < 3; ++k) { e.v[k] = W.v[k]; e.vL[k] = vL[k]; }
	e.vSq = vSq;
	e.hTotal = hTotal;
	e.Cs = Cs;
}

// The edge assignment of the revision that recorded the reference's 'plm-athena'
// errors (tests/test-order/schemes.lua:104,117-126): L from the left-edge
// value, R from the right-edge value.  With it the oracle reproduces those
// recorded errors; the current source (the default, 0) swaps the two.
static int g_plmAthenaRecordedEdges = 0;

// "plm athena", the first of the two branches of that name
// (hydro/solver/plm.cl:782-879; the second, :950-968, is never reached): the
// primitive differences are projected with the cell's eigenvectors of the
// conserved system, limited per wave, projected back, clamped to the
// neighbouring primitives, and stored with the reference's assignment: the
// cell's L state from the right-edge value and its R state from the
// left-edge value (plm.cl:877-878) unless g_plmAthenaRecordedEdges is set.
static void plmAthena(cons_t& L, cons_t& R, const Solver& s, const cons_t& UL, const cons_t& U, const cons_t& UR,
		int side) {
	eigen_t eig;
	eigen_forCell(eig, s, U);
	prim_t W, WL, WR;
	primFromCons(W, s, U);
	primFromCons(WL, s, UL);
	primFromCons(WR, s, UR);
	real dWL[6], dWR[6], dWC[6], dWG[6];
	for (int j = 0; j < 5; ++j) {
		dWL[j] = primAt(W, j) - primAt(WL, j);
		dWR[j] = primAt(WR, j) - primAt(W, j);
		dWC[j] = .5 * (primAt(WR, j) - primAt(WL, j));
		dWG[j] = (dWL[j] * dWR[j]) <= 0. ? 0. : (2. * dWL[j] * dWR[j] / (dWL[j] + dWR[j]));
	}
	dWL[5] = dWR[5] = dWC[5] = dWG[5] = 0.;
	real dal[5], dar[5], dac[5], dag[5];
	eigen_leftTransform(dal, s, eig, dWL, side);
	eigen_leftTransform(dar, s, eig, dWR, side);
	eigen_leftTransform(dac, s, eig, dWC, side);
	eigen_leftTransform(dag, s, eig, dWG, side);
	real da[5];
	for (int j = 0; j < 5; ++j) {
		da[j] = 0;
		if (dal[j] * dar[j] > 0) {
			real const lim_slope1 = clMin(std::fabs(dal[j]), std::fabs(dar[j]));
			real const lim_slope2 = clMin(std::fabs(dac[j]), std::fabs(dag[j]));
			da[j] = clSign(dac[j]) * clMin((real)2. * lim_slope1, lim_slope2);
		}
	}
	real dWm[6];
	eigen_rightTransform(dWm, s, eig, da, side);
	prim_t Wlv = W, Wrv = W;
	for (int j = 0; j < 5; ++j) {
		real const w = primAt(W, j), wl = primAt(WL, j), wr = primAt(WR, j);
		real lv = w - .5 * dWm[j];
		real rv = w + .5 * dWm[j];
		real const C = rv + lv;
		lv = clMax(clMin(w, wl), lv);
		lv = clMin(clMax(w, wl), lv);
		rv = C - lv;
		rv = clMax(clMin(w, wr), rv);
		rv = clMin(clMax(w, wr), rv);
		lv = C - rv;
		primAt(Wlv, j) = lv;
		primAt(Wrv, j) = rv;
	}
	if (g_plmAthenaRecordedEdges) {
		consFromPrim(L, s, Wlv);
		consFromPrim(R, s, Wrv);
	} else {
		consFromPrim(L, s, Wrv);
		consFromPrim(R, s, Wlv);
	}
}

// hydro/solver/plm.cl:976-997 (calcLR over [1, n-1) on every axis);
// "piecewise constant" copies the cell (plm.cl:10-25)
static void calcLR(Solver& s) {
	forAllCells(s, [&](const int* i, long index) {
		if (OOB(s, i, 1, 1)) return;
		const cons_t& U = s.U[index];
		for (int side = 0; side < s.dim; ++side) {
			cons_t& L = s.ULR[2 * (side + s.dim * index) + 0];
			cons_t& R = s.ULR[2 * (side + s.dim * index) + 1];
			const cons_t& UL = s.U[index - s.stepsize[side]];
			const cons_t& UR = s.U[index + s.stepsize[side]];
			switch (s.recon) {
			case RECON_PLM_CONS: plmCons(L, R, s, UL, U, UR); break;
			case RECON_PLM_PRIM: plmPrim(L, R, s, UL, U, UR); break;
			case RECON_PLM_ATHENA: plmAthena(L, R, s, UL, U, UR, side); break;
			default: L = U; R = U; break;
			}
		}
	});
}

// hydro/solver/fvsolver.lua:55-199
static void calcFlux(Solver& s, real dt) {
	int const G = Solver::numGhost;
	bool const usePLM = s.recon != RECON_NONE;
	// only the Roe flux takes the flux limiter (fvsolver.lua:62-64, flux.usesFluxLimiter)
	bool const useFluxLimiter = s.fluxLimiter > 0 && s.fluxType == FLUX_ROE;
	forAllCells(s, [&](const int* i, long index) {
		if (OOB(s, i, G, G - 1)) return;
		long const indexR = index;
		for (int side = 0; side < s.dim; ++side) {
			real const dx = s.grid_dx[side];
			long const indexL = index - s.stepsize[side];
			cons_t& flux = s.flux[side + s.dim * index];
			real area = 1.;
			for (int k = 0; k < s.dim; ++k) if (k != side) area = area * s.grid_dx[k];
			if (area <= 1e-7) {
				for (int j = 0; j < 6; ++j) flux.ptr[j] = 0;
				continue;
			}
			auto lr = [&](long iL, long iR, const cons_t*& pUL, const cons_t*& pUR) {
				if (usePLM) {
					pUL = &s.ULR[2 * (side + s.dim * iL) + 1];  // .R of the left cell
					pUR = &s.ULR[2 * (side + s.dim * iR) + 0];  // .L of the right cell
				} else {
					pUL = &s.U[iL];
					pUR = &s.U[iR];
				}
			};
			const cons_t *UL, *UR, *UL_L = 0, *UR_L = 0, *UL_R = 0, *UR_R = 0;
			lr(indexL, indexR, UL, UR);
			real dt_dx = 0;
			if (useFluxLimiter) {
				dt_dx = dt / dx;
				long const indexR2 = indexR + s.stepsize[side];
				long const indexL2 = indexL - s.stepsize[side];
				lr(indexL2, indexL, UL_L, UR_L);
				lr(indexR, indexR2, UL_R, UR_R);
			}
			if (s.fluxType == FLUX_HLL) hllFluxForInterface(flux, s, *UL, *UR, side);
			else if (s.fluxType == FLUX_HLLC) hllcFluxForInterface(flux, s, *UL, *UR, side);
			else if (s.fluxType == FLUX_RUSANOV) rusanovFluxForInterface(flux, s, *UL, *UR, side);
			else roeFluxForInterface(flux, s, *UL, *UR, side, useFluxLimiter, dt_dx, UL_L, UL_R, UR_L, UR_R);
		}
	});
}

// hydro/solver/fvsolver.cl:6-125 (holonomic / Cartesian branch)
static void calcDerivFromFlux(Solver& s, std::vector<cons_t>& deriv) {
	int const G = Solver::numGhost;
	forAllCells(s, [&](const int* i, long index) {
		if (OOB(s, i, G, G)) return;
		real volume = 1.;
		for (int k = 0; k < s.dim; ++k) volume = volume * s.grid_dx[k];
		cons_t& d = deriv[index];
		for (int side = 0; side < s.dim; ++side) {
			const cons_t& fluxL = s.flux[side + s.dim * index];
			const cons_t& fluxR = s.flux[side + s.dim * (index + s.stepsize[side])];
			real areaL = 1.;
			for (int k = 0; k < s.dim; ++k) if (k != side) areaL = areaL * s.grid_dx[k];
			real areaR = areaL;
			if (volume > 1e-7) {
				real const invVolume = 1. / volume;
				if (areaL <= 1e-7) areaL = 0.;
				if (areaR <= 1e-7) areaR = 0.;
				areaL *= invVolume;
				areaR *= invVolume;
				for (int j = 0; j < 5; ++j)
					d.ptr[j] -= fluxR.ptr[j] * areaR - fluxL.ptr[j] * areaL;
			}
		}
	});
}

// hydro/solver/fvsolver.lua:225-302
static void calcDeriv(Solver& s, std::vector<cons_t>& deriv, real dt) {
	if (s.recon != RECON_NONE) calcLR(s);
	calcFlux(s, dt);
	calcDerivFromFlux(s, deriv);
}

static void clearBuffer(std::vector<cons_t>& b) { std::memset(b.data(), 0, b.size() * sizeof(cons_t)); }

// hydro/solver/solverbase.lua:1216-1251 (interior only)
static void multAddInto(Solver& s, std::vector<cons_t>& a, const std::vector<cons_t>& b, real c) {
	int const G = Solver::numGhost;
	forAllCells(s, [&](const int* i, long index) {
		if (OOB(s, i, G, G)) return;
		for (int j = 0; j < 5; ++j) a[index].ptr[j] += b[index].ptr[j] * c;
	});
}
static void multAdd(Solver& s, std::vector<cons_t>& a, const std::vector<cons_t>& b, const std::vector<cons_t>& c, real d) {
	int const G = Solver::numGhost;
	forAllCells(s, [&](const int* i, long index) {
		if (OOB(s, i, G, G)) return;
		for (int j = 0; j < 5; ++j) a[index].ptr[j] = b[index].ptr[j] + c[index].ptr[j] * d;
	});
}

// hydro/int/fe.lua:33-49
static void integrateFE(Solver& s, real dt) {
	std::vector<cons_t>& deriv = s.derivs[0];
	clearBuffer(deriv);
	calcDeriv(s, deriv, dt);
	multAddInto(s, s.U, deriv, dt);
	boundary(s);
	constrainU(s);
}

// hydro/int/rk.lua:47-167
static void integrateRK(Solver& s, real dt) {
	const RKTable& T = rkTables[s.integrator];
	int const order = T.order;
	auto alphaNeeded = [&](int i) { bool n = false; for (int m = i; m <= order; ++m) n = n || T.alpha[m - 1][i - 1] != 0; return n; };
	auto betaNeeded = [&](int i) { bool n = false; for (int m = i; m <= order; ++m) n = n || T.beta[m - 1][i - 1] != 0; return n; };
	if (alphaNeeded(1)) s.UBufs[0] = s.U;
	if (betaNeeded(1)) {
		clearBuffer(s.derivs[0]);
		calcDeriv(s, s.derivs[0], dt);
	}
	for (int i = 2; i <= order + 1; ++i) {
		clearBuffer(s.U);
		for (int k = 1; k <= i - 1; ++k)
			if (T.alpha[i - 2][k - 1] != 0) multAdd(s, s.U, s.U, s.UBufs[k - 1], T.alpha[i - 2][k - 1]);
		for (int k = 1; k <= i - 1; ++k)
			if (T.beta[i - 2][k - 1] != 0) multAdd(s, s.U, s.U, s.derivs[k - 1], T.beta[i - 2][k - 1] * dt);
		boundary(s);
		constrainU(s);
		if (i <= order) {
			if (alphaNeeded(i)) s.UBufs[i - 1] = s.U;
			if (betaNeeded(i)) {
				clearBuffer(s.derivs[i - 1]);
				calcDeriv(s, s.derivs[i - 1], dt);
			}
		}
	}
}

// hydro/eqn/cl/calcDT.cl:38-73 + hydro/eqn/eqn.lua:1182-1235 + solverbase.lua:3004-3024
static real calcDT(Solver& s) {
	if (s.fixedDT > 0) return s.fixedDT;
	int const G = Solver::numGhost;
	forAllCells(s, [&](const int* i, long index) {
		real dt = INFINITY;
		if (!OOB(s, i, G, G)) {
			const cons_t& U = s.U[index];
			real const Cs = calc_Cs_fromCons(s, U);
			for (int side = 0; side < s.dim; ++side) {
				real const dx = s.grid_dx[side];
				if (dx > 0) {
					real const Cs_nLen = Cs * 1.;
					real const v_n = U.ptr[0] < s.rhoMin ? 0. : U.ptr[1 + side] / U.ptr[0];
					real const lambdaMin = v_n - Cs_nLen;
					real const lambdaMax = v_n + Cs_nLen;
					real absLambdaMax = cl_max(std::fabs(lambdaMin), std::fabs(lambdaMax));
					absLambdaMax = cl_max((real)1e-9, absLambdaMax);
					dt = cl_min(dt, dx / absLambdaMax);
				}
			}
		}
		s.dtBuf[index] = dt;
	});
	real m = INFINITY;
	for (long k = 0; k < s.numCells; ++k) m = std::min(m, s.dtBuf[k]);
	return s.cfl * m;
}

static void step(Solver& s, real dt) {
	if (s.integrator == 0) integrateFE(s, dt);
	else integrateRK(s, dt);
}

// hydro/solver/solverbase.lua:3026-3190
static real update(Solver& s) {
	real const dt = calcDT(s);
	step(s, dt);
	s.t = s.t + dt;
	boundary(s);
	return dt;
}

} // namespace

// ---------------------------------------------------------------------------
// C interface for the tests (ctypes)
// ---------------------------------------------------------------------------

extern "C" {

typedef struct or_desc {
	int dim;
	int n[3];
	double mins[3];
	double maxs[3];
	int boundary[6];
	int flux_limiter;
	int recon;
	int slope_limiter;
	int integrator;
	double gamma;
	double rho_min;
	double p_min;
	double cfl;
	double fixed_dt;
	int flux;          // FLUX_*: roe, hll, rusanov, euler-hllc
	int hllc_method;   // 0: the reference's default (its hllcMethod 2); 1, 2, 3: its hllcMethod 0, 1, 2
	int entropy_fix;   // Roe: useEntropyFluxFix
	int reserved0;
	double entropy_fix_factor;
	double fixed_cons[6][5];   // BC_FIXED sides
} or_desc;

void* or_create(const or_desc* d) {
	if (d->dim < 1 || d->dim > 3 || d->integrator < 0 || d->integrator >= numIntegrators) return 0;
	Solver* s = new Solver();
	s->dim = d->dim;
	for (int k = 0; k < 3; ++k) {
		s->n[k] = k < d->dim ? d->n[k] : 1;
		s->gs[k] = k < d->dim ? d->n[k] + 2 * Solver::numGhost : 1;
		s->mins[k] = d->mins[k];
		s->maxs[k] = d->maxs[k];
		s->grid_dx[k] = (d->maxs[k] - d->mins[k]) / (double)s->n[k];
	}
	s->stepsize[0] = 1;
	s->stepsize[1] = s->gs[0];
	s->stepsize[2] = s->gs[0] * s->gs[1];
	s->numCells = (long)s->gs[0] * s->gs[1] * s->gs[2];
	for (int k = 0; k < 6; ++k) s->bc[k] = d->boundary[k];
	s->fluxLimiter = d->flux_limiter;
	s->fluxType = d->flux;
	s->hllcMethod = d->hllc_method == 0 ? 2 : d->hllc_method - 1;
	s->recon = d->recon;
	s->slopeLimiter = d->slope_limiter;
	s->integrator = d->integrator;
	s->gamma = d->gamma;
	s->rhoMin = d->rho_min;
	s->PMin = d->p_min;
	s->cfl = d->cfl;
	s->fixedDT = d->fixed_dt;
	s->entropyFix = d->entropy_fix != 0;
	s->entropyFactor = d->entropy_fix_factor;
	for (int k = 0; k < 6; ++k)
		for (int f = 0; f < 5; ++f) s->fixedCons[k][f] = d->fixed_cons[k][f];
	s->t = 0;
	s->U.assign(s->numCells, cons_t{});
	s->ULR.assign(2 * s->numCells * s->dim, cons_t{});
	s->flux.assign(s->numCells * s->dim, cons_t{});
	s->dtBuf.assign(s->numCells, 0.);
	int const order = s->integrator == 0 ? 1 : rkTables[s->integrator].order;
	for (int k = 0; k < order; ++k) {
		s->UBufs[k].assign(s->numCells, cons_t{});
		s->derivs[k].assign(s->numCells, cons_t{});
	}
	return s;
}

void or_destroy(void* h) { delete (Solver*)h; }

long or_num_cells(void* h) { return ((Solver*)h)->numCells; }

// Full AoS-6 buffer with ghosts (numCells * 6 doubles).
void or_set_state_full(void* h, const double* src) {
	Solver& s = *(Solver*)h;
	std::memcpy(s.U.data(), src, s.numCells * sizeof(cons_t));
}
void or_get_state_full(void* h, double* dst) {
	Solver& s = *(Solver*)h;
	std::memcpy(dst, s.U.data(), s.numCells * sizeof(cons_t));
}

// resetState after applyInitCond (solverbase.lua:2094-2114): the caller's
// AoS-6 interior state is written, then boundary and constrainU.
void or_reset_state(void* h, const double* interior) {
	Solver& s = *(Solver*)h;
	int const G = Solver::numGhost;
	std::fill(s.U.begin(), s.U.end(), cons_t{});
	long k = 0;
	for (int z = 0; z < s.n[2]; ++z) for (int y = 0; y < s.n[1]; ++y) for (int x = 0; x < s.n[0]; ++x, ++k) {
		int c[3] = { x + (s.dim > 0 ? G : 0), y + (s.dim > 1 ? G : 0), z + (s.dim > 2 ? G : 0) };
		std::memcpy(s.U[INDEX(s, c[0], c[1], c[2])].ptr, interior + 6 * k, sizeof(cons_t));
	}
	s.t = 0;
	boundary(s);
	constrainU(s);
}

void or_get_interior(void* h, double* dst) {
	Solver& s = *(Solver*)h;
	int const G = Solver::numGhost;
	long k = 0;
	for (int z = 0; z < s.n[2]; ++z) for (int y = 0; y < s.n[1]; ++y) for (int x = 0; x < s.n[0]; ++x, ++k) {
		int c[3] = { x + (s.dim > 0 ? G : 0), y + (s.dim > 1 ? G : 0), z + (s.dim > 2 ? G : 0) };
		std::memcpy(dst + 6 * k, s.U[INDEX(s, c[0], c[1], c[2])].ptr, sizeof(cons_t));
	}
}

void or_boundary(void* h) { boundary(*(Solver*)h); }
void or_constrain_u(void* h) { constrainU(*(Solver*)h); }
double or_calc_dt(void* h) { return calcDT(*(Solver*)h); }
void or_step(void* h, double dt) { step(*(Solver*)h, dt); }
double or_update(void* h) { return update(*(Solver*)h); }
double or_get_t(void* h) { return ((Solver*)h)->t; }
void or_set_t(void* h, double t) { ((Solver*)h)->t = t; }

// App loop (hydro/app.lua:1573-1600): stop when t >= exitTime, checked before
// each update, so the final step overshoots.  Returns the number of updates.
long or_run_until(void* h, double t_end, long max_steps) {
	Solver& s = *(Solver*)h;
	long k = 0;
	while (!(s.t >= t_end) && k < max_steps) { update(s); ++k; }
	return k;
}

// One calcDeriv into a zeroed buffer (numCells * 6 doubles), for kernel-level checks.
void or_calc_deriv(void* h, double dt, double* deriv_out) {
	Solver& s = *(Solver*)h;
	std::vector<cons_t> d(s.numCells, cons_t{});
	calcDeriv(s, d, dt);
	std::memcpy(deriv_out, d.data(), s.numCells * sizeof(cons_t));
}

// Flux buffer after the last calcFlux (numCells * dim * 6 doubles).
void or_get_flux(void* h, double* dst) {
	Solver& s = *(Solver*)h;
	std::memcpy(dst, s.flux.data(), s.flux.size() * sizeof(cons_t));
}

// Single-interface Roe flux, for unit checks.
// The interface flux of the descriptor's flux function (roe without a limiter, hll, rusanov).
void or_interface_flux(const or_desc* d, const double* UL, const double* UR, int side, double* out) {
	Solver* s = (Solver*)or_create(d);
	cons_t a, b, f;
	std::memcpy(a.ptr, UL, sizeof(a));
	std::memcpy(b.ptr, UR, sizeof(b));
	std::memset(f.ptr, 0, sizeof(f));
	if (d->flux == FLUX_HLL) hllFluxForInterface(f, *s, a, b, side);
	else if (d->flux == FLUX_HLLC) hllcFluxForInterface(f, *s, a, b, side);
	else if (d->flux == FLUX_RUSANOV) rusanovFluxForInterface(f, *s, a, b, side);
	else roeFluxForInterface(f, *s, a, b, side, false, 0, 0, 0, 0, 0);
	std::memcpy(out, f.ptr, sizeof(f));
	delete s;
}

void or_roe_flux(const or_desc* d, const double* UL, const double* UR, int side, double* out) {
	Solver* s = (Solver*)or_create(d);
	cons_t a, b, f;
	std::memcpy(a.ptr, UL, sizeof(a));
	std::memcpy(b.ptr, UR, sizeof(b));
	roeFluxForInterface(f, *s, a, b, side, false, 0, 0, 0, 0, 0);
	std::memcpy(out, f.ptr, sizeof(f));
	delete s;
}

// Interface eigen-basis: left (5x5) and right (5x5) matrices at the Roe state
// of (UL, UR), column by column, plus the 5 wave speeds.  Used to check
// L.R = I and R.diag(lambda).L = A (hydro/solver/fvsolver.lua:396-527).
void or_eigen_basis(const or_desc* d, const double* UL, const double* UR, int side,
                    double* Lmat, double* Rmat, double* lambdas) {
	Solver* s = (Solver*)or_create(d);
	cons_t a, b;
	std::memcpy(a.ptr, UL, sizeof(a));
	std::memcpy(b.ptr, UR, sizeof(b));
	eigen_t e;
	eigen_forInterface(e, *s, a, b);
	for (int c = 0; c < 5; ++c) {
		real X[6] = {0, 0, 0, 0, 0, 0};
		X[c] = 1;
		real w[5];
		eigen_leftTransform(w, *s, e, X, side);
		for (int r = 0; r < 5; ++r) Lmat[r * 5 + c] = w[r];
		real Y[5] = {0, 0, 0, 0, 0};
		Y[c] = 1;
		real u[6];
		eigen_rightTransform(u, *s, e, Y, side);
		for (int r = 0; r < 5; ++r) Rmat[r * 5 + c] = u[r];
	}
	lambdas[0] = e.v[side] - e.Cs;
	lambdas[1] = lambdas[2] = lambdas[3] = e.v[side];
	lambdas[4] = e.v[side] + e.Cs;
	delete s;
}

double or_limiter(int which, double r) { return limiter(which, r); }

// 1: "plm athena" with the recorded revision's edge assignment; 0: the current source's
void or_set_plm_athena_recorded_edges(int on) { g_plmAthenaRecordedEdges = on ? 1 : 0; }

int or_num_threads(void) {
#ifdef _OPENMP
	return omp_get_max_threads();
#else
	return 1;
#endif
}

} // extern "C"
