// physics.cuh — per-particle material models shared by the FP64 and mixed-precision pair loops.
//
//   TillotsonEos / IdealGasEos::evaluate (core/physics/Eos.cpp:42-45, 198-238)
//   VonMisesRheology::initialize (core/physics/Rheology.cpp:36-83)
//   findEigenvalues (core/objects/geometry/SymmetricTensor.h:377-398) for ScalarGradyKippModel::integrate
//   AdaptiveSmoothingLength::initialize (core/sph/equations/EquationTerm.cpp:356-364)
//   clampWithDerivative (core/objects/wrappers/Interval.h:159-162)
#pragma once

#include <cfloat>

#include "state.h"

namespace sphgpu {
namespace {

// Fast (the mixed-precision path): the same expressions with the reciprocals of the material constants, of the
// density and of the denominator formed once and the divisions turned into products (FP64 results that differ in
// the last bits); the FP64 path keeps the reference's divisions.
template <bool Fast>
__device__ void eosEvalT(const MaterialD& mt, double rho, double u, double& p, double& cs) {
    if (mt.eos == SPHGPU_EOS_IDEAL_GAS) {
        const double gamma = mt.gamma;
        p = (gamma - 1.) * u * rho;
        cs = sqrt(gamma * p / rho);
        return;
    }
    const double rho0 = mt.rho0, A = mt.A, B = mt.B, a = mt.a, b = mt.b, alpha = mt.alpha, beta = mt.beta;
    const double u0 = mt.u0, uiv = mt.uiv, ucv = mt.ucv;
    const double eta = Fast ? rho * mt.inv_rho0 : rho / rho0;
    const double mu = eta - 1.;
    const double denom = Fast ? u * mt.inv_u0 * (1. / (eta * eta)) + 1. : u / (u0 * eta * eta) + 1.;
    const double invDen = Fast ? 1. / denom : 0.;
    const double invDen2 = invDen * invDen;
    const double invRho = Fast ? 1. / rho : 0.;
    const double invRho2 = invRho * invRho;
    const double pc = (Fast ? a + b * invDen : a + b / denom) * rho * u + A * mu + B * mu * mu;
    double dpdu = Fast ? a * rho + b * rho * invDen2 : a * rho + b * rho / (denom * denom);
    double dpdrho = Fast ? a * u + b * u * (3. * denom - 2.) * invDen2 + A * mt.inv_rho0 + 2. * B * mu * mt.inv_rho0
                         : a * u + b * u * (3. * denom - 2.) / (denom * denom) + A / rho0 + 2. * B * mu / rho0;
    const double csc = Fast ? dpdrho + dpdu * pc * invRho2 : dpdrho + dpdu * pc / (rho * rho);
    double pp = pc, cc = csc;
    // the expanded phase enters only for rho <= rho0 above the incipient / complete vaporisation energies; it is
    // formed only then (the reference forms it always and uses it only then: the same values)
    const bool vapor = rho <= rho0 && u > ucv;
    const bool blend = rho <= rho0 && u > uiv && u <= ucv;
    if (vapor || blend) {
        const double rhoExp = Fast ? rho0 * invRho - 1. : rho0 / rho - 1.;
        const double betaExp = exp(-fmin(beta * rhoExp, 70.));
        const double alphaExp = exp(-fmin(alpha * (rhoExp * rhoExp), 70.));
        double pe, cse;
        if (Fast) {
            pe = a * rho * u + (b * rho * u * invDen + A * mu * betaExp) * alphaExp;
            dpdu = a * rho + alphaExp * b * rho * invDen2;
            dpdrho = a * u + alphaExp * (b * u * (3. * denom - 2.) * invDen2) +
                     alphaExp * (b * u * rho * invDen) * rho0 * (2. * alpha * rhoExp) * invRho2 +
                     alphaExp * A * betaExp * (mt.inv_rho0 + rho0 * mu * invRho2 * (2. * alpha * rhoExp + beta));
            cse = dpdrho + dpdu * pe * invRho2;
        } else {
            pe = a * rho * u + (b * rho * u / denom + A * mu * betaExp) * alphaExp;
            dpdu = a * rho + alphaExp * b * rho / (denom * denom);
            dpdrho = a * u + alphaExp * (b * u * (3. * denom - 2.) / (denom * denom)) +
                     alphaExp * (b * u * rho / denom) * rho0 * (2. * alpha * rhoExp) / (rho * rho) +
                     alphaExp * A * betaExp * (1. / rho0 + rho0 * mu / (rho * rho) * (2. * alpha * rhoExp + beta));
            cse = dpdrho + dpdu * pe / (rho * rho);
        }
        cse = fmax(cse, 0.);
        if (vapor) {
            pp = pe;
            cc = cse;
        } else {
            pp = ((u - uiv) * pe + (ucv - u) * pc) / (ucv - uiv);
            cc = ((u - uiv) * cse + (ucv - u) * csc) / (ucv - uiv);
        }
    }
    cc = fmax(cc, Fast ? 0.25 * A * mt.inv_rho0 : 0.25 * A / rho0);
    p = pp;
    cs = sqrt(cc);
}

__device__ __forceinline__ double ddotTT(const double s[5], const double t[5]) {
    const double szz = -s[0] - s[1], tzz = -t[0] - t[1];
    return (s[0] * t[0] + s[1] * t[1] + szz * tzz) + 2. * (s[2] * t[2] + s[3] * t[3] + s[4] * t[4]);
}

// sqrtApprox of the reference (core/math/MathUtils.h:42-62): float inverse square root with one Newton
// step, used only as the normalisation of the eigenvalue solver
__device__ double sqrtApproxRef(double f) {
    if (f == 0.) {
        return 0.;
    }
    const float x2 = __fmul_rn(float(f), 0.5f);
    float y = float(f);
    int i = __float_as_int(y);
    i = 0x5f3759df - (i >> 1);
    y = __int_as_float(i);
    const float t = __fsub_rn(1.5f, __fmul_rn(__fmul_rn(x2, y), y));
    return 1. / double(__fmul_rn(y, t));
}

// findEigenvalues (core/objects/geometry/SymmetricTensor.h:377-398); t = xx yy zz xy xz yz
__device__ void eigenvalues(const double t[6], double sig[3]) {
    const double dx = t[0], dy = t[1], dz = t[2], ox = t[3], oy = t[4], oz = t[5];
    const double mx = fmax(dx, ox), my = fmax(dy, oy), mz = fmax(dz, oz);
    const double n = sqrtApproxRef(mx * mx + my * my + mz * mz);
    if (n < 1.e-12) {
        sig[0] = sig[1] = sig[2] = 0.;
        return;
    }
    const double inv1 = dx * 1. + dy * 1. + dz * 1.;
    const double inv2 = (ox * ox + oy * oy + oz * oz) - (dy * dz + dz * dx + dx * dy);
    const double inv3 = dx * dy * dz + 2. * ox * oy * oz - ((ox * ox) * dz + (oy * oy) * dy + (oz * oz) * dx);
    const double p = -inv1 / n;
    const double q = -inv2 / (n * n);
    const double r = -inv3 / (n * n * n);
    const double a = q - p * p / 3.;
    const double b = (2. * (p * p * p) - 9. * p * q + 27. * r) / 27.;
    const double aCub = (a * a * a) / 27.;
    if (0.25 * b * b + aCub >= 0.) {
        sig[0] = sig[1] = sig[2] = 0.;
        return;
    }
    const double t1 = 2. * sqrt(-a / 3.);
    const double phi = acos(-0.5 * b / sqrt(-aCub));
    const double p3 = p / 3.;
    sig[0] = (t1 * cos(phi / 3.) - p3) * n;
    sig[1] = (t1 * cos((phi + 2. * SPH_PI) / 3.) - p3) * n;
    sig[2] = (t1 * cos((phi + 4. * SPH_PI) / 3.) - p3) * n;
}

// The largest eigenvalue of findEigenvalues' result for the mixed-precision path: the same characteristic
// polynomial in FP64 with the divisions by constants and by the norm turned into products, and only the root
// of cos(phi / 3), which is the largest for phi in [0, pi] (the reference forms all three roots and takes the
// largest: the same value up to the last bits). The acos argument is clamped to [-1, 1] against rounding.
__device__ double maxEigenvalueFast(const double t[6]) {
    const double dx = t[0], dy = t[1], dz = t[2], ox = t[3], oy = t[4], oz = t[5];
    const double mx = fmax(dx, ox), my = fmax(dy, oy), mz = fmax(dz, oz);
    const double n = sqrtApproxRef(mx * mx + my * my + mz * mz);
    if (n < 1.e-12) {
        return 0.;
    }
    const double invN = 1. / n;
    const double inv1 = dx + dy + dz;
    const double inv2 = (ox * ox + oy * oy + oz * oz) - (dy * dz + dz * dx + dx * dy);
    const double inv3 = dx * dy * dz + 2. * ox * oy * oz - ((ox * ox) * dz + (oy * oy) * dy + (oz * oz) * dx);
    const double p = -inv1 * invN;
    const double q = -inv2 * (invN * invN);
    const double r = -inv3 * (invN * invN * invN);
    const double a = q - p * p * (1. / 3.);
    const double b = (2. * (p * p * p) - 9. * p * q + 27. * r) * (1. / 27.);
    const double aCub = (a * a * a) * (1. / 27.);
    if (0.25 * b * b + aCub >= 0.) {
        return 0.;
    }
    const double t1 = 2. * sqrt(-a * (1. / 3.));
    const double phi = acos(fmin(fmax(-0.5 * b * rsqrt(-aCub), -1.), 1.));
    return (t1 * cos(phi * (1. / 3.)) - p * (1. / 3.)) * n;
}

// AdaptiveSmoothingLength::initialize (core/sph/equations/EquationTerm.cpp:356-364): h clamped to its range.
// Applied with the position update, before the tree build reads h as the gravitational softening.
__device__ __forceinline__ void clampSmoothingLength(const DState& s, const Physics& ph, uint32_t i) {
    if (ph.adaptive_h) {
        dbl4 r = s.r[i];
        r.w = fmax(ph.h_lo, fmin(r.w, ph.h_hi));
        s.r[i] = r;
    }
}

// materials initialize (EOS, von Mises) for particle i; does not read h. Fast: the mixed path (eosEvalT<true>,
// products by the reciprocals of u_melt and of sqrt(3 J2))
template <bool Fast>
__device__ void materialInit(const DState& s, const Physics& ph, const MaterialD* __restrict__ mats, uint32_t i) {
    const MaterialD mt = mats[ph.nmat > 1 ? s.mat[i] : 0];
    double p, cs;
    eosEvalT<Fast>(mt, s.rho[i], s.u[i], p, cs);
    if (ph.solid && mt.yielding != SPHGPU_YIELDING_NONE) {
        const uint32_t n = s.n;
        const double d = (s.D && mt.damage != SPHGPU_DAMAGE_NONE) ? s.D[i] * s.D[i] * s.D[i] : 0.;
        if (p < 0.) {
            p = (1. - d) * p;
        }
        const double unorm = Fast ? s.u[i] * mt.inv_u_melt : s.u[i] / mt.u_melt;
        double Y = unorm < 1.e-5 ? mt.limit : mt.limit * fmax(1. - unorm, 0.);
        Y = (1. - d) * Y;
        double S[5];
        for (int c = 0; c < 5; ++c) {
            S[c] = s.S[c * n + i];
        }
        if (Y < SPH_EPS) {
            s.reduce[i] = 0.;
            for (int c = 0; c < 5; ++c) {
                s.S[c * n + i] = 0.;
            }
        } else {
            const double J2 = 0.5 * ddotTT(S, S) + 1.e-15;
            const double red = fmin(Fast ? Y * rsqrt(3. * J2) : Y / sqrt(3. * J2), 1.);
            s.reduce[i] = red;
            for (int c = 0; c < 5; ++c) {
                s.S[c * n + i] = S[c] * red;
            }
        }
    }
    s.p[i] = p;
    s.cs[i] = cs;
}

// clampWithDerivative (core/objects/wrappers/Interval.h:159-162)
__device__ __forceinline__ void clampDeriv(double& x, double& dx, double lo, double hi) {
    if (lo == -DBL_MAX && hi == DBL_MAX) {
        return;
    }
    const bool zero = (x >= hi && dx > 0.) || (x <= lo && dx < 0.);
    x = fmax(lo, fmin(x, hi));
    if (zero) {
        dx = 0.;
    }
}


// EquationHolder::finalize in reverse term order (core/sph/equations/EquationTerm.h:293-297):
// AdaptiveSmoothingLength / ConstSmoothingLength (EquationTerm.cpp:366-391, 427-434), ContinuityEquation
// (:289-316), SolidStressForce (:177-203), PressureForce (:90-99); then the fracture model of the material
// (ScalarGradyKippModel::integrate, core/physics/Damage.cpp:128-170). Writes every highest derivative of
// particle i from the pair sums (the reference zeroes them before the loop). Fast (the mixed-precision path):
// the same terms with the divisions by constants and the repeated reciprocals of the density turned into
// products and the largest principal stress from maxEigenvalueFast (results that differ in the last FP64 bits);
// the FP64 path keeps the reference's operations.
template <bool Solid, bool Fast = false>
__device__ __forceinline__ void finalizeParticle(const DState& s, const Physics& ph, const MaterialD* __restrict__ mats,
    uint32_t i, const dbl4& ri, double rhoi, double pri, const double Si[5], double ax, double ay, double az,
    double du, double divv, const double gv[6], uint32_t cnt) {
    const uint32_t n = s.n;
    const MaterialD mt = mats[ph.nmat > 1 ? s.mat[i] : 0];
    const double invRho = Fast ? 1. / rhoi : 0.;
    dbl4 vout = s.v[i];
    if (ph.adaptive_h) {
        vout.w = ri.w > 2. * ph.h_lo ? (Fast ? ri.w * (1. / 3.) * divv : ri.w / 3. * divv) : 0.;
    } else {
        vout.w = 0.;
    }
    s.v[i] = vout;
    s.dv[i] = mkd4(ax, ay, az, 0.);
    s.divv[i] = divv;
    s.ncnt[i] = cnt;
    s.drho[i] = 0. + -rhoi * divv;
    if (Solid) {
        for (int c = 0; c < 6; ++c) {
            s.gradv[c * n + i] = gv[c];
        }
        double dS[5] = { 0, 0, 0, 0, 0 };
        if (mt.yielding != SPHGPU_YIELDING_NONE) {
            const double szz = -Si[0] - Si[1];
            du += (Fast ? invRho : 1. / rhoi) * ((Si[0] * gv[0] + Si[1] * gv[1] + szz * gv[2]) +
                                                    2. * (Si[2] * gv[3] + Si[3] * gv[4] + Si[4] * gv[5]));
            const double tr3 = Fast ? (gv[0] + gv[1] + gv[2]) * (1. / 3.) : (gv[0] * 1. + gv[1] * 1. + gv[2] * 1.) / 3.;
            const double twoMu = 2. * mt.mu;
            dS[0] = 0. + twoMu * (gv[0] - tr3);
            dS[1] = 0. + twoMu * (gv[1] - tr3);
            dS[2] = 0. + twoMu * gv[3];
            dS[3] = 0. + twoMu * gv[4];
            dS[4] = 0. + twoMu * gv[5];
        }
        for (int c = 0; c < 5; ++c) {
            s.dS[c * n + i] = dS[c];
        }
    }
    du -= (Fast ? pri * invRho : pri / rhoi) * divv;
    s.du[i] = du;
    if (Solid && ph.damage) {
        double dD = 0.;
        if (mt.yielding != SPHGPU_YIELDING_NONE && mt.damage == SPHGPU_DAMAGE_SCALAR_GRADY_KIPP) {
            const double D = s.D[i];
            if (D >= mt.d_hi) {
                dD = SPH_LARGE;
            } else {
                const double sigma[6] = { Si[0] - pri, Si[1] - pri, (-Si[0] - Si[1]) - pri, Si[2], Si[3], Si[4] };
                double sigMax;
                if (Fast) {
                    sigMax = maxEigenvalueFast(sigma);
                } else {
                    double sig[3];
                    eigenvalues(sigma, sig);
                    sigMax = fmax(fmax(sig[0], sig[1]), sig[2]);
                }
                const double youngRed = fmax((1. - D * D * D) * mt.young, 1.e-20);
                const double ratio = Fast ? sigMax / (youngRed * s.eps_min[i]) : (sigMax / youngRed) / s.eps_min[i];
                if (ratio > 1.) {
                    dD = s.growth[i] * cbrt(fmin(pow(ratio, s.m_zero[i]), double(s.n_flaws[i])));
                }
            }
        }
        s.dD[i] = dD;
    }
}

} // namespace
} // namespace sphgpu
